// Inverse BWT of a batch of blocks by LF-mapping on sm_103a.
//
// Replaces the inverse transform libbsc runs inside bsc_decompress after QLFC
// decoding (reached from crates/qz-lib/src/compression/bsc.rs:421-433).
//
// Block b has n_b + 1 rows (row 0 = the empty suffix, row p_b = the whole
// block, whose last-column symbol is the dropped sentinel).  Rows of all
// blocks are stored back to back: block b's rows start at off[b] + b.
//
//   1. LF build: a stable ranking of U by symbol per block (per-tile 8-bit
//      histograms, one device-wide scan, warp match-based ranks), so
//      LF[row] = 1 + (number of symbols < c) + (occurrences of c before row);
//   2. list ranking of the single LF cycle with rulers, the rows r with
//      r % stride == 0:
//      - walk 1: each ruler walks LF to the next ruler, and stages the
//        first-column symbol F(row) of the rows it passes (the output bytes of
//        its stretch, in walk order) in a fixed-capacity slot of its own;
//      - the ruler list is ranked with a second ruling set: every 32nd ruler of
//        a block is a head; heads walk the ruler list to the next head, the
//        head list is ranked by pointer jumping, and each head walks its ruler
//        segment again handing every ruler its distance to row 0;
//      - each ruler's staged bytes are copied to T[n - d - t] (one warp per
//        ruler, coalesced), and only a walk longer than the slot re-reads LF,
//        from the row where its staging stopped.
// So every LF row is read once (plus the tails of long walks), and every wait
// is a bounded loop: a broken LF cycle (corrupt input) is reported as
// QZGPU_DATA_CORRUPT for its block.
#include <algorithm>
#include <mutex>

#include "engine.h"
#include "scan.cuh"

namespace qz {

constexpr int kIRItems = kInitTile / kThreads;  // 16
constexpr int kIRWarpSpan = kInitTile / kWarps;  // 512
constexpr int kHeadLog2 = 5;                     // a head every 32 rulers

struct InvArgs {
    const uint8_t* U;
    const int* off;
    const int* idx;
    const int* tbase;  // first histogram tile of each block
    const int* rbase;  // first ruler of each block
    const int2* tiles; // (block, start) per kInitTile tile of U
    int* LF;
    int stride_log2;
    DevStatus* st;
    int* bst;          // per-block status (may be null)
};

// Per-tile symbol counts (order-independent): per-warp shared counters with
// atomics, all of the tile's bytes loaded first.
__global__ void __launch_bounds__(kThreads) k_inv_up(InvArgs a, uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[kWarps][256];
#pragma unroll
    for (int q = 0; q < kWarps; ++q) h[q][threadIdx.x] = 0;
    __syncthreads();
    int2 tl = a.tiles[blockIdx.x];
    int b = tl.x, s0 = tl.y;
    int bs = a.off[b], n = a.off[b + 1] - bs;
    int j = (s0 - bs) / kInitTile;
    int m = (n + kInitTile - 1) / kInitTile;
    int end = min(bs + n, s0 + kInitTile);
    unsigned cu[kInitTile / kThreads];
#pragma unroll
    for (int it = 0; it < kInitTile / kThreads; ++it) {
        int x = s0 + it * kThreads + threadIdx.x;
        cu[it] = x < end ? (unsigned)__ldg(a.U + x) : 256u;
    }
#pragma unroll
    for (int it = 0; it < kInitTile / kThreads; ++it)
        if (cu[it] < 256u) atomicAdd(&h[warp_id()][cu[it]], 1u);
    __syncthreads();
    uint32_t v = 0;
#pragma unroll
    for (int q = 0; q < kWarps; ++q) v += h[q][threadIdx.x];
    hist[(size_t)256 * a.tbase[b] + (size_t)threadIdx.x * m + j] = v;
}

__global__ void __launch_bounds__(kThreads) k_inv_down(InvArgs a, const uint32_t* __restrict__ hist) {
    __shared__ uint32_t wcnt[kWarps][256];
    __shared__ uint32_t base_of[256];
    const unsigned w = warp_id(), ln = lane_id();
    int2 tl = a.tiles[blockIdx.x];
    int b = tl.x, s0 = tl.y;
    int bs = a.off[b], n = a.off[b + 1] - bs;
    int j = (s0 - bs) / kInitTile;
    int m = (n + kInitTile - 1) / kInitTile;
    int cnt = min(kInitTile, bs + n - s0);
    int p = a.idx[b];
    int* LF = a.LF + bs + b;  // rows of this block
#pragma unroll
    for (int q = 0; q < kWarps; ++q) wcnt[q][threadIdx.x] = 0;
    __syncthreads();
    uint8_t cc[kIRItems];
    uint32_t rk[kIRItems];
    unsigned cu[kIRItems];
    // all of the tile's symbols in flight at once, then the ranking; full
    // tiles without per-slot predicates
    if (cnt == kInitTile) {
#pragma unroll
        for (int it = 0; it < kIRItems; ++it) cu[it] = (unsigned)__ldg(a.U + s0 + (int)w * kIRWarpSpan + it * 32 + (int)ln);
#pragma unroll
        for (int it = 0; it < kIRItems; ++it) {
            cc[it] = (uint8_t)cu[it];
            rk[it] = warp_digit_rank(cu[it], true, wcnt[w]);
        }
    } else {
#pragma unroll
        for (int it = 0; it < kIRItems; ++it) {
            int i = (int)w * kIRWarpSpan + it * 32 + (int)ln;
            cu[it] = i < cnt ? (unsigned)__ldg(a.U + s0 + i) : 0u;
        }
#pragma unroll
        for (int it = 0; it < kIRItems; ++it) {
            int i = (int)w * kIRWarpSpan + it * 32 + (int)ln;
            cc[it] = (uint8_t)cu[it];
            rk[it] = warp_digit_rank(cu[it], i < cnt, wcnt[w]);
        }
    }
    __syncthreads();
    {
        unsigned c = threadIdx.x;
        uint32_t run = 0;
#pragma unroll
        for (int q = 0; q < kWarps; ++q) {
            uint32_t v = wcnt[q][c];
            wcnt[q][c] = run;
            run += v;
        }
        // rows before this tile's first c within the block, plus the sentinel row 0
        base_of[c] = hist[(size_t)256 * a.tbase[b] + (size_t)c * m + j] - (uint32_t)bs + 1u;
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < kIRItems; ++it) {
        int i = (int)w * kIRWarpSpan + it * 32 + (int)ln;
        if (i < cnt) {
            unsigned c = cc[it];
            int u = s0 - bs + i;
            int row = u < p ? u : u + 1;
            LF[row] = (int)(base_of[c] + wcnt[w][c] + rk[it]);
        }
    }
    if (j == 0 && threadIdx.x == 0) LF[p] = 0;
}

// Rulers of all blocks, indexed back to back (block b's from rbase[b]); heads
// likewise from hbase[b].
struct RulerArgs {
    const int2* rtiles;  // (block, first local ruler) per CTA
    int* next0;          // ruler reached by walking LF from this one (-1: row 0)
    int* len;            // rows walked to reach it
    int* distF;          // rows from this ruler's row to row 0 along the cycle (ranked)
    const int* hbase;    // first head of each block
    int* hnext;          // head: next head on the list (-1: row 0), rows to reach it
    int* hdist;
    uint8_t* stage;      // cap bytes per ruler: F of the rows a walk passes (null if cap == 0)
    int* resume;         // row at step cap of a walk longer than cap
    int cap;             // bytes staged per ruler (a multiple of 16, or 0)
};

// First-column symbol table of block b in shared memory: C[i] = first row of
// the i-th present symbol (1 + count of smaller symbols), C[sigma] = n + 1,
// sym[i] = that symbol.  Every thread of the CTA takes part; returns sigma.
__device__ __forceinline__ int load_first_column(const uint32_t* __restrict__ hist, const int* __restrict__ tbase,
                                                 int b, int bs, int n, int* C, uint8_t* sym, int* s_cnt) {
    const int m = (n + kInitTile - 1) / kInitTile;
    const uint32_t* hb = hist + (size_t)256 * tbase[b];
    const int c0 = (int)(hb[(size_t)threadIdx.x * m] - (uint32_t)bs) + 1;
    const int c1 = threadIdx.x < 255 ? (int)(hb[(size_t)(threadIdx.x + 1) * m] - (uint32_t)bs) + 1 : n + 1;
    const bool present = c1 > c0;
    int tot;
    const int at = block_excl_sum(present ? 1 : 0, s_cnt, &tot);
    if (present) {
        C[at] = c0;
        sym[at] = (uint8_t)threadIdx.x;
    }
    if (threadIdx.x == 0) {
        C[tot] = n + 1;
        s_cnt[kWarps] = tot;
    }
    __syncthreads();
    return s_cnt[kWarps];
}

// F(row): the symbol whose first-column range holds `row` (log2 sigma steps).
__device__ __forceinline__ unsigned first_col(const int* C, const uint8_t* sym, int sigma, int row) {
    int lo = 0, hi = sigma - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (C[mid] <= row) lo = mid; else hi = mid - 1;
    }
    return sym[lo];
}

// Walk 1: each ruler follows LF to the next ruler, staging F of the rows it
// passes (first `cap` of them, 16 bytes per store) and the row where staging
// stopped.  The next row's load is issued before the symbol search.
__global__ void __launch_bounds__(kThreads) k_inv_walk1(InvArgs a, RulerArgs r, const uint32_t* __restrict__ hist) {
    __shared__ int C[257];
    __shared__ uint8_t sym[256];
    __shared__ int s_cnt[kWarps + 1];
    const int2 rt = r.rtiles[blockIdx.x];
    const int b = rt.x;
    const int bs = a.off[b], n = a.off[b + 1] - bs;
    const int sigma = r.cap ? load_first_column(hist, a.tbase, b, bs, n, C, sym, s_cnt) : 1;
    const int mask = (1 << a.stride_log2) - 1;
    const int M = (n >> a.stride_log2) + 1;
    const int lq = rt.y + threadIdx.x;
    if (lq >= M) return;
    const int* LF = a.LF + bs + b;
    const int q = a.rbase[b] + lq;
    const int cap = r.cap;
    uint4* stage = r.cap ? reinterpret_cast<uint4*>(r.stage + (size_t)q * cap) : nullptr;
    int cur = lq << a.stride_log2;
    int steps = 0;
    bool ok = true;
    // staged bytes: w fills a word, a0..a3 the 16 bytes of the next store
    uint32_t w = 0, a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    const unsigned long long pol = l2_keep_policy();
    do {
        const int nxt = ld_keep(LF + cur, pol);
        if (steps < cap) {
            w |= first_col(C, sym, sigma, cur) << (8 * (steps & 3));
            if ((steps & 3) == 3) {
                const int k = (steps >> 2) & 3;
                a0 = k == 0 ? w : a0;
                a1 = k == 1 ? w : a1;
                a2 = k == 2 ? w : a2;
                a3 = k == 3 ? w : a3;
                w = 0;
                if (k == 3) stage[steps >> 4] = make_uint4(a0, a1, a2, a3);
            }
        } else if (steps == cap && cap) {
            r.resume[q] = cur;
        }
        cur = nxt;
        ++steps;
        if (cur < 0 || cur > n || steps > n + 1) {
            ok = false;
            break;
        }
    } while (cur & mask);
    if (!ok) {
        report_block(a.st, a.bst, QZGPU_DATA_CORRUPT, 10, b);
        r.next0[q] = -1;
        r.len[q] = 0;
        return;
    }
    const int kept = min(steps, cap);
    if (kept & 15) {  // the last, partly filled 16 bytes (only `kept` bytes are ever read)
        const int k = (kept >> 2) & 3;
        if (kept & 3) {
            a0 = k == 0 ? w : a0;
            a1 = k == 1 ? w : a1;
            a2 = k == 2 ? w : a2;
            a3 = k == 3 ? w : a3;
        }
        stage[kept >> 4] = make_uint4(a0, a1, a2, a3);
    }
    const int nl = cur >> a.stride_log2;
    r.next0[q] = nl == 0 ? -1 : a.rbase[b] + nl;
    r.len[q] = steps;
}

// Heads (every 32nd ruler of a block, ruler 0 first): walk the ruler list to
// the next head, summing the rows.  One thread per ruler; the heads work.
__global__ void __launch_bounds__(kThreads) k_inv_heads(InvArgs a, RulerArgs r) {
    const int2 rt = r.rtiles[blockIdx.x];
    const int b = rt.x;
    const int n = a.off[b + 1] - a.off[b];
    const int M = (n >> a.stride_log2) + 1;
    const int lq = rt.y + threadIdx.x;
    if (lq >= M || (lq & ((1 << kHeadLog2) - 1))) return;
    const int rb = a.rbase[b];
    const int h = r.hbase[b] + (lq >> kHeadLog2);
    int q = rb + lq, d = 0, steps = 0;
    do {
        d += r.len[q];
        q = r.next0[q];
        ++steps;
    } while (q >= 0 && ((q - rb) & ((1 << kHeadLog2) - 1)) && steps <= M);
    if (steps > M) {  // a cycle of rulers that never reaches row 0
        report_block(a.st, a.bst, QZGPU_DATA_CORRUPT, 14, b);
        q = -1;
    }
    r.hnext[h] = q < 0 ? -1 : r.hbase[b] + ((q - rb) >> kHeadLog2);
    r.hdist[h] = d;
}

// Heads, once ranked (hdist = rows to row 0): each walks its ruler segment
// again, giving every ruler its own distance to row 0.
__global__ void __launch_bounds__(kThreads) k_inv_spread(InvArgs a, RulerArgs r, const int* __restrict__ hdist) {
    const int2 rt = r.rtiles[blockIdx.x];
    const int b = rt.x;
    const int n = a.off[b + 1] - a.off[b];
    const int M = (n >> a.stride_log2) + 1;
    const int lq = rt.y + threadIdx.x;
    if (lq >= M || (lq & ((1 << kHeadLog2) - 1))) return;
    const int rb = a.rbase[b];
    int d = hdist[r.hbase[b] + (lq >> kHeadLog2)];
    int q = rb + lq, steps = 0;
    do {
        r.distF[q] = d;
        d -= r.len[q];
        q = r.next0[q];
        ++steps;
    } while (q >= 0 && ((q - rb) & ((1 << kHeadLog2) - 1)) && steps <= M);
}

// Output offset of ruler q's stretch: its first byte goes to T[n - d0], the
// next ones downwards.  Checks what corrupt input could break; returns -1 then.
__device__ __forceinline__ int ruler_start(const InvArgs& a, const RulerArgs& r, int b, int n, int lq, int q) {
    const int D = r.distF[q];
    // ruler 0's list covers the whole cycle exactly when LF is one cycle
    if (D < 0 || D > n + 1 || (lq == 0 && D != n + 1)) return -1;
    return (n + 1) - D;
}

// Staged bytes to their places.  A warp takes 32 consecutive rulers: lane l
// loads ruler l's length and distance (coalesced), then the warp copies the
// rulers' runs one after the other, lane t taking byte t (a run is contiguous,
// so a warp's stores are).
__global__ void __launch_bounds__(kThreads) k_inv_place(InvArgs a, RulerArgs r, int nb, int Mtot,
                                                        uint8_t* __restrict__ T) {
    const int ln = (int)lane_id();
    const int nwarps = gridDim.x * kWarps;
    for (int q0 = (blockIdx.x * kWarps + (int)warp_id()) * 32; q0 < Mtot; q0 += nwarps * 32) {
        const int q = q0 + ln;
        int L = 0, d0 = -1, bs = 0, n = 0, b = 0;
        if (q < Mtot) {
            b = block_of(a.rbase, nb, q);
            bs = __ldg(a.off + b);
            n = __ldg(a.off + b + 1) - bs;
            L = r.len[q];
            d0 = ruler_start(a, r, b, n, q - __ldg(a.rbase + b), q);
            if (d0 < 0) report_block(a.st, a.bst, QZGPU_DATA_CORRUPT, 11, b);
        }
        const int last = min(32, Mtot - q0);
        for (int k = 0; k < last; ++k) {
            const int Lk = __shfl_sync(0xffffffffu, L, k), dk = __shfl_sync(0xffffffffu, d0, k);
            const int bsk = __shfl_sync(0xffffffffu, bs, k), nk = __shfl_sync(0xffffffffu, n, k);
            const int bk = __shfl_sync(0xffffffffu, b, k);
            if (dk < 0) continue;  // uniform across the warp
            const int m = min(Lk, r.cap);
            const uint8_t* src = r.stage + (size_t)(q0 + k) * r.cap;
            for (int t = ln; t < m; t += 32) {
                const int s = nk - dk - t;
                if (s >= nk) continue;  // row 0: the sentinel, no output byte
                if (s < 0) {
                    report_block(a.st, a.bst, QZGPU_DATA_CORRUPT, 13, bk);
                    break;
                }
                T[bsk + s] = src[t];
            }
        }
    }
}

// The part of each walk that staging did not hold (all of it when cap == 0):
// walk LF again from the row where staging stopped, writing T[n - d0 - t] =
// F(row).  Bytes are packed into 32-bit words aligned on their address, so a
// run leaves as word stores; a word this walk does not fill is stored byte by
// byte.
__global__ void __launch_bounds__(kThreads) k_inv_walk2(InvArgs a, RulerArgs r, const uint32_t* __restrict__ hist,
                                                        uint8_t* __restrict__ T) {
    __shared__ int C[257];
    __shared__ uint8_t sym[256];
    __shared__ int s_cnt[kWarps + 1];
    const int2 rt = r.rtiles[blockIdx.x];
    const int b = rt.x;
    const int bs = a.off[b], n = a.off[b + 1] - bs;
    const int sigma = load_first_column(hist, a.tbase, b, bs, n, C, sym, s_cnt);
    const int M = (n >> a.stride_log2) + 1;
    const int lq = rt.y + threadIdx.x;
    if (lq >= M) return;
    const int q = a.rbase[b] + lq;
    const int L = r.len[q];
    if (L <= r.cap) return;  // staged whole
    const int d0 = ruler_start(a, r, b, n, lq, q);
    if (d0 < 0) {
        if (!r.cap) report_block(a.st, a.bst, QZGPU_DATA_CORRUPT, 12, b);  // else reported by k_inv_place
        return;
    }
    const int* LF = a.LF + bs + b;
    int cur = r.cap ? r.resume[q] : (lq << a.stride_log2);
    if (cur < 0 || cur > n) {
        report_block(a.st, a.bst, QZGPU_DATA_CORRUPT, 15, b);
        return;
    }
    uint8_t* out = T + bs;
    const unsigned long long pol = l2_keep_policy();
    uintptr_t word_at = 0;  // address of the word being filled (0: none)
    uint32_t word = 0;
    unsigned have = 0;      // bytes of that word filled so far (bit mask)
    auto flush = [&]() {
        if (!have) return;
        if (have == 0xfu) {
            *reinterpret_cast<uint32_t*>(word_at) = word;
        } else {
            for (int k = 0; k < 4; ++k)
                if (have & (1u << k)) reinterpret_cast<uint8_t*>(word_at)[k] = (uint8_t)(word >> (8 * k));
        }
    };
    for (int t = r.cap; t < L; ++t) {
        // the next row is loaded first; the symbol search below overlaps it
        const int nxt = ld_keep(LF + cur, pol);
        const int s = n - d0 - t;
        if (s < 0) {
            report_block(a.st, a.bst, QZGPU_DATA_CORRUPT, 13, b);
            return;
        }
        if (s < n) {
            const unsigned c = first_col(C, sym, sigma, cur);
            uintptr_t addr = reinterpret_cast<uintptr_t>(out + s);
            uintptr_t wa = addr & ~(uintptr_t)3;
            if (wa != word_at) {
                flush();
                word_at = wa;
                word = 0;
                have = 0;
            }
            int k = (int)(addr & 3);
            word |= c << (8 * k);
            have |= 1u << k;
        }
        cur = nxt;
        if (cur < 0 || cur > n) {
            report_block(a.st, a.bst, QZGPU_DATA_CORRUPT, 15, b);
            return;
        }
    }
    flush();
}

// One pointer-jumping step over all rulers: dist += dist[next], next = next[next].
__global__ void __launch_bounds__(kThreads) k_inv_jump(int M, const int* __restrict__ nin,
                                                       const int* __restrict__ din, int* __restrict__ nout,
                                                       int* __restrict__ dout) {
    for (int q = blockIdx.x * kThreads + threadIdx.x; q < M; q += gridDim.x * kThreads) {
        int nx = nin[q];
        int d = din[q];
        if (nx >= 0) {
            d += din[nx];
            nx = nin[nx];
        }
        nout[q] = nx;
        dout[q] = d;
    }
}

namespace {

// Bytes staged per ruler: 4 per row of the stride, so a walk up to four times
// the mean length needs no second pass (a 16-byte multiple).
int stage_cap(int stride_log2) { return 4 << stride_log2; }

}  // namespace

size_t inverse_stage_bytes(long long cap_bytes, int cap_blocks) {
    // sum over blocks of rulers * cap <= 4 * (n_b + stride) at the largest stride (2^12)
    return 4 * (size_t)cap_bytes + (size_t)stage_cap(12) * (size_t)(cap_blocks + 1);
}

namespace {

// The inverse of one batch.  chained: tables go to the area the chain fills
// next (after that area's previous copies have run), the device status is
// left to the chain, and the call returns once the work is queued.
int inverse_issue(Storage* S, int nb, const int* n, const int* idx, const uint8_t* d_U, uint8_t* d_T,
                  cudaStream_t st, int* block_rc, bool chained) {
    if (nb < 0 || nb > S->cap_blocks) return QZGPU_BAD_PARAMETER;
    long long N = 0;
    for (int b = 0; b < nb; ++b) {
        if (n[b] < 0) return QZGPU_BAD_PARAMETER;
        N += n[b];
    }
    if (block_rc)
        for (int b = 0; b < nb; ++b) block_rc[b] = 0;
    for (int b = 0; b < nb; ++b) {
        if (n[b] > 0 && (idx[b] < 1 || idx[b] > n[b])) {
            if (block_rc) block_rc[b] = QZGPU_DATA_CORRUPT;
            return QZGPU_DATA_CORRUPT;  // before any launch: no block is inverted
        }
    }
    if (N > S->cap_bytes) return QZGPU_BAD_PARAMETER;
    S->stats = qzgpu_stats{};
    S->launches = 0;
    if (N == 0) return QZGPU_NO_ERROR;
    const int stride_log2 = S->tune.ruler_log2;  // rulers every 2^stride_log2 rows
    const int stride = 1 << stride_log2;
    const int cap = stage_cap(stride_log2);

    std::vector<int> off(nb + 1, 0), tbase(nb + 1, 0), rbase(nb + 1, 0), hbase(nb + 1, 0);
    std::vector<int2> tiles, rtiles;
    int maxH = 1;
    for (int b = 0; b < nb; ++b) {
        off[b + 1] = off[b] + n[b];
        int m = (n[b] + kInitTile - 1) / kInitTile;
        tbase[b + 1] = tbase[b] + m;
        for (int s = off[b]; s < off[b + 1]; s += kInitTile) tiles.push_back(make_int2(b, s));
        int M = n[b] > 0 ? n[b] / stride + 1 : 0;
        rbase[b + 1] = rbase[b] + M;
        int H = (M + (1 << kHeadLog2) - 1) >> kHeadLog2;
        hbase[b + 1] = hbase[b] + H;
        for (int q = 0; q < M; q += kThreads) rtiles.push_back(make_int2(b, q));
        if (H > maxH) maxH = H;
    }
    const int Mtot = rbase[nb], Htot = hbase[nb];
    if ((size_t)tbase[nb] * 256 > S->hist_cap) return QZGPU_BAD_PARAMETER;
    size_t need = sizeof(int) * (5 * (nb + 1)) + sizeof(int2) * (tiles.size() + rtiles.size()) + 256;
    if (need > S->pin_tab_bytes) return QZGPU_BAD_PARAMETER;
    const int slot = S->tab_slot;
    if (chained) {
        // the copies that last read this area must have run before it is refilled
        const cudaError_t w = cudaEventSynchronize(S->tab_ev[slot]);
        if (w != cudaSuccess) return map_cuda_error(w);
    }
    char* p = chained && slot ? S->pin_tab_alt : S->pin_tab;
    auto put = [&](const void* src, size_t bytes) {
        char* at = p;
        if (bytes) memcpy(p, src, bytes);
        p += (bytes + 15) / 16 * 16;
        return at;
    };
    char* h_off = put(off.data(), sizeof(int) * off.size());
    char* h_idx = put(idx, sizeof(int) * nb);
    char* h_tb = put(tbase.data(), sizeof(int) * tbase.size());
    char* h_rb = put(rbase.data(), sizeof(int) * rbase.size());
    char* h_hb = put(hbase.data(), sizeof(int) * hbase.size());
    char* h_tiles = put(tiles.data(), sizeof(int2) * tiles.size());
    char* h_rt = put(rtiles.data(), sizeof(int2) * rtiles.size());
    cudaError_t e = cudaSuccess;
    auto h2d = [&](void* dst, const char* src, size_t bytes) {
        if (bytes && e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    };
    InvBuffers& v = S->v;
    h2d(S->blk_off, h_off, sizeof(int) * off.size());
    h2d(S->blk_idx, h_idx, sizeof(int) * nb);
    h2d(S->blk_tbase, h_tb, sizeof(int) * tbase.size());
    h2d(S->blk_aux_off, h_rb, sizeof(int) * rbase.size());  // ruler bases reuse this table
    h2d(S->blk_hbase, h_hb, sizeof(int) * hbase.size());
    h2d(S->tiles, h_tiles, sizeof(int2) * tiles.size());
    h2d(v.rtiles, h_rt, sizeof(int2) * rtiles.size());
    if (chained && e == cudaSuccess) {
        e = cudaEventRecord(S->tab_ev[slot], st);
        S->tab_slot = slot ^ 1;
    }
    if (!chained && e == cudaSuccess) e = cudaMemsetAsync(S->status, 0, sizeof(DevStatus), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(S->blk_status, 0, sizeof(int) * nb, st);
    // a ruler no head reaches (corrupt input) keeps -1 and is reported
    if (e == cudaSuccess) e = cudaMemsetAsync(v.distF, 0xff, sizeof(int) * Mtot, st);
    if (e != cudaSuccess) return map_cuda_error(e);

    InvArgs a{d_U, S->blk_off, S->blk_idx, S->blk_tbase, S->blk_aux_off, S->tiles, v.LF, stride_log2, S->status,
              S->blk_status};
    RulerArgs r{v.rtiles, v.next0, v.len, v.distF, S->blk_hbase, v.hnext[0], v.hdist[0], v.stage, v.resume, cap};
    const int ntiles = (int)tiles.size();
    const int hist_len = tbase[nb] * 256;
    const long long rows = N + nb;
    const int nrt = (int)rtiles.size();
    // U read once for the histogram, once for the ranks; LF written once
    QZ_LAUNCH(S, st, "k_inv_up", N, k_inv_up<<<ntiles, kThreads, 0, st>>>(a, S->hist));
    scan_exclusive(S, S->hist, S->hist, hist_len, nullptr, nullptr, st);
    QZ_LAUNCH(S, st, "k_inv_down", 5 * N, k_inv_down<<<ntiles, kThreads, 0, st>>>(a, S->hist));
    // every row's LF entry read once, one byte staged per row; 8 bytes per ruler
    QZ_LAUNCH(S, st, "k_inv_walk1", 5 * rows + 8ll * Mtot, k_inv_walk1<<<nrt, kThreads, 0, st>>>(a, r, S->hist));
    // heads: ruler list read (8 bytes per ruler), 8 bytes per head written
    QZ_LAUNCH(S, st, "k_inv_heads", 8ll * Mtot + 8ll * Htot, k_inv_heads<<<nrt, kThreads, 0, st>>>(a, r));
    int cur = 0;
    const int jgrid = (int)std::min<long long>(((long long)Htot + kThreads - 1) / kThreads, (long long)S->sms * 16);
    for (long long span = 1; span < maxH + 1; span <<= 1) {
        QZ_LAUNCH(S, st, "k_inv_jump", 24ll * Htot,
                  k_inv_jump<<<jgrid, kThreads, 0, st>>>(Htot, v.hnext[cur], v.hdist[cur], v.hnext[cur ^ 1],
                                                          v.hdist[cur ^ 1]));
        cur ^= 1;
    }
    // heads again: ruler list read, every ruler's distance written
    QZ_LAUNCH(S, st, "k_inv_spread", 12ll * Mtot, k_inv_spread<<<nrt, kThreads, 0, st>>>(a, r, v.hdist[cur]));
    // staged bytes read and written once
    const int pgrid = (int)std::min<long long>(((long long)Mtot + 32 * kWarps - 1) / (32 * kWarps), (long long)S->sms * 16);
    QZ_LAUNCH(S, st, "k_inv_place", 2 * N + 12ll * Mtot,
              k_inv_place<<<pgrid, kThreads, 0, st>>>(a, r, nb, Mtot, d_T));
    // walks longer than the staging slot: their tails only
    QZ_LAUNCH(S, st, "k_inv_walk2", 12ll * Mtot, k_inv_walk2<<<nrt, kThreads, 0, st>>>(a, r, S->hist, d_T));
    if (chained) {
        S->stats.kernel_launches = S->launches;
        S->stats.alg_bytes = 12 * N;
        return map_cuda_error(cudaGetLastError());
    }
    DevStatus* hst = reinterpret_cast<DevStatus*>(S->pin_rd);
    int* hbs = S->pin_rd + 64;  // per-block results (pinned; nb <= cap_blocks entries fit)
    e = cudaMemcpyAsync(hst, S->status, sizeof(DevStatus), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && block_rc) e = cudaMemcpyAsync(hbs, S->blk_status, sizeof(int) * nb, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return map_cuda_error(e);
    prof_flush(S);
    if (hst->error) {
        if (debug_on()) debug_log("device status %d at %d detail %lld", hst->error, hst->where, hst->detail);
        if (block_rc) {
            // every corrupt-data report names its block; any other failure
            // leaves no block's result trusted
            bool named = false;
            for (int b = 0; b < nb; ++b) {
                block_rc[b] = hbs[b];
                named |= hbs[b] != 0;
            }
            if (hst->error != QZGPU_DATA_CORRUPT || !named)
                for (int b = 0; b < nb; ++b) block_rc[b] = hst->error;
        }
        return hst->error;
    }
    S->stats.kernel_launches = S->launches;
    S->stats.alg_bytes = 12 * N;
    return QZGPU_NO_ERROR;
}

}  // namespace

int inverse_run(Storage* S, int nb, const int* n, const int* idx, const uint8_t* d_U, uint8_t* d_T,
                cudaStream_t st, int* block_rc) {
    return inverse_issue(S, nb, n, idx, d_U, d_T, st, block_rc, false);
}

int inverse_run_chained(Storage* S, int nb, const int* n, const int* idx, const uint8_t* d_U, uint8_t* d_T,
                        cudaStream_t st) {
    return inverse_issue(S, nb, n, idx, d_U, d_T, st, nullptr, true);
}

void inverse_chain_begin(Storage* S, cudaStream_t st) {
    cudaMemsetAsync(S->status, 0, sizeof(DevStatus), st);
    S->inv_chained = true;
}

int inverse_chain_end(Storage* S, cudaStream_t st) {
    S->inv_chained = false;
    DevStatus* hst = reinterpret_cast<DevStatus*>(S->pin_rd);
    cudaError_t e = cudaMemcpyAsync(hst, S->status, sizeof(DevStatus), cudaMemcpyDeviceToHost, st);
    const cudaError_t w = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = w;
    if (e != cudaSuccess) return map_cuda_error(e);
    prof_flush(S);
    if (hst->error && debug_on())
        debug_log("device status %d at %d detail %lld", hst->error, hst->where, hst->detail);
    return hst->error;
}

}  // namespace qz

// ------------------------------------------------------------------ allocation-free inverse
//
// For callers that cannot allocate device memory while they run: a pipeline
// stage inside a host runtime that owns every device allocation up front
// (and forbids cudaMalloc/cudaFree later), or code on a thread that must not
// take the allocator's locks.  The caller passes device input and output;
// all scratch of the inverse lives in one file-scope array below, sized for
// blocks of up to QZGPU_NOALLOC_MAX_BLOCK bytes.  It runs the kernels above
// without staging (every walk writes its bytes on its second pass).

namespace qz {
namespace noalloc {

constexpr long long kMaxN = QZGPU_NOALLOC_MAX_BLOCK;
constexpr long long kMaxTiles = (kMaxN + kInitTile - 1) / kInitTile;
constexpr int kStrideLog2 = 5;
constexpr long long kMaxRulers = (kMaxN >> kStrideLog2) + 1;
constexpr long long kMaxHeads = (kMaxRulers + (1 << kHeadLog2) - 1) >> kHeadLog2;
constexpr long long kMaxRTiles = (kMaxRulers + kThreads - 1) / kThreads;

constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }
// byte offsets inside the scratch array
constexpr size_t kOffLF = 0;
constexpr size_t kOffHist = align256(kOffLF + 4 * (kMaxN + 2));
constexpr size_t kOffPartial = align256(kOffHist + 4 * 256 * kMaxTiles);
constexpr size_t kOffRuler = align256(kOffPartial + 4 * 1024);
constexpr size_t kRulerBytes = align256(4 * kMaxRulers);
constexpr size_t kOffHeads = kOffRuler + 3 * kRulerBytes;  // next0, len, distF
constexpr size_t kHeadBytes = align256(4 * kMaxHeads);
constexpr size_t kOffTiles = kOffHeads + 4 * kHeadBytes;   // hnext, hdist, twice
constexpr size_t kOffRTiles = align256(kOffTiles + 8 * kMaxTiles);
constexpr size_t kOffTables = align256(kOffRTiles + 8 * kMaxRTiles);  // off, idx, tbase, rbase, hbase
constexpr size_t kOffStatus = align256(kOffTables + 4 * 16);
constexpr size_t kBytes = align256(kOffStatus + sizeof(DevStatus));
static_assert(kBytes <= (6u << 20), "allocation-free scratch exceeds its stated 6 MiB");

}  // namespace noalloc

// Every GPU that loads this library holds this array until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[noalloc::kBytes];

// Per-block tables of a single-block inverse, built on the device; ruler
// distances cleared (a ruler no head reaches keeps -1).
__global__ void k_noalloc_tables(char* scratch, int n, int index) {
    using namespace noalloc;
    int* tab = reinterpret_cast<int*>(scratch + kOffTables);
    int m = (n + kInitTile - 1) / kInitTile;
    int M = (n >> kStrideLog2) + 1;
    int H = (M + (1 << kHeadLog2) - 1) >> kHeadLog2;
    if (threadIdx.x == 0) {
        tab[0] = 0;  // off
        tab[1] = n;
        tab[2] = index;  // idx
        tab[4] = 0;      // tbase
        tab[5] = m;
        tab[6] = 0;      // rbase
        tab[7] = M;
        tab[8] = 0;      // hbase
        tab[9] = H;
        *reinterpret_cast<DevStatus*>(scratch + kOffStatus) = DevStatus{0, 0, 0};
    }
    int2* tiles = reinterpret_cast<int2*>(scratch + kOffTiles);
    for (int j = threadIdx.x; j < m; j += blockDim.x) tiles[j] = make_int2(0, j * kInitTile);
    int2* rtiles = reinterpret_cast<int2*>(scratch + kOffRTiles);
    int nrt = (M + kThreads - 1) / kThreads;
    for (int j = threadIdx.x; j < nrt; j += blockDim.x) rtiles[j] = make_int2(0, j * kThreads);
    int* distF = reinterpret_cast<int*>(scratch + kOffRuler + 2 * kRulerBytes);
    for (int j = threadIdx.x; j < M; j += blockDim.x) distF[j] = -1;
}

namespace {

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[256];

// Device address of the scratch array for the current device, looked up once
// per device (host code must not use the array's name as a device address).
// The address belongs to the device's primary context: a cudaDeviceReset in
// the process invalidates it, and calls after such a reset are not supported
// (as for every storage this library holds).
int noalloc_scratch(char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return map_cuda_error(e);
    if (dev < 0 || dev >= 256) return QZGPU_GPU_NOT_SUPPORTED;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return map_cuda_error(e == cudaSuccess ? cudaErrorInvalidSymbol : e);
        g_noalloc_ptr[dev] = p;
    }
    *out = static_cast<char*>(g_noalloc_ptr[dev]);
    return QZGPU_NO_ERROR;
}

}  // namespace

}  // namespace qz

extern "C" int qzgpu_bwt_decode_noalloc(const unsigned char* d_U, unsigned char* d_T, int n, int index,
                                        void* stream) {
    using namespace qz;
    using namespace qz::noalloc;
    if (n < 0 || (n > 0 && (!d_U || !d_T))) return QZGPU_BAD_PARAMETER;
    if (n > QZGPU_NOALLOC_MAX_BLOCK) return QZGPU_BLOCK_TOO_LARGE;
    if (n == 0) return QZGPU_NO_ERROR;
    if (index < 1 || index > n) return QZGPU_DATA_CORRUPT;
    // an error left by the caller's own earlier work is not this call's: it
    // stays for the caller to read (peek does not clear it) and nothing runs
    if (cudaPeekAtLastError() != cudaSuccess) return QZGPU_GPU_ERROR;
    char* sc = nullptr;
    int rc = noalloc_scratch(&sc);
    if (rc) return rc;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    int* tab = reinterpret_cast<int*>(sc + kOffTables);
    const int m = (n + kInitTile - 1) / kInitTile;
    const int M = (n >> kStrideLog2) + 1;
    const int H = (M + (1 << kHeadLog2) - 1) >> kHeadLog2;
    const int nrt = (M + kThreads - 1) / kThreads;
    int* next0 = reinterpret_cast<int*>(sc + kOffRuler);
    int* len = reinterpret_cast<int*>(sc + kOffRuler + kRulerBytes);
    int* distF = reinterpret_cast<int*>(sc + kOffRuler + 2 * kRulerBytes);
    int* hn[2] = {reinterpret_cast<int*>(sc + kOffHeads), reinterpret_cast<int*>(sc + kOffHeads + kHeadBytes)};
    int* hd[2] = {reinterpret_cast<int*>(sc + kOffHeads + 2 * kHeadBytes),
                  reinterpret_cast<int*>(sc + kOffHeads + 3 * kHeadBytes)};
    uint32_t* hist = reinterpret_cast<uint32_t*>(sc + kOffHist);
    DevStatus* dst = reinterpret_cast<DevStatus*>(sc + kOffStatus);

    // launch bookkeeping for the shared scan helper only; it owns no memory
    Storage ctx;
    ctx.partial = reinterpret_cast<uint32_t*>(sc + kOffPartial);

    k_noalloc_tables<<<1, kThreads, 0, st>>>(sc, n, index);
    InvArgs a{d_U, tab, tab + 2, tab + 4, tab + 6, reinterpret_cast<const int2*>(sc + kOffTiles),
              reinterpret_cast<int*>(sc + kOffLF), kStrideLog2, dst};
    k_inv_up<<<m, kThreads, 0, st>>>(a, hist);
    scan_exclusive(&ctx, hist, hist, 256 * m, nullptr, nullptr, st);
    k_inv_down<<<m, kThreads, 0, st>>>(a, hist);
    RulerArgs r{reinterpret_cast<const int2*>(sc + kOffRTiles), next0, len, distF, tab + 8, hn[0], hd[0],
                nullptr, nullptr, 0};
    k_inv_walk1<<<nrt, kThreads, 0, st>>>(a, r, hist);
    k_inv_heads<<<nrt, kThreads, 0, st>>>(a, r);
    int cur = 0;
    for (long long span = 1; span < (long long)H + 1; span <<= 1) {
        k_inv_jump<<<(H + kThreads - 1) / kThreads, kThreads, 0, st>>>(H, hn[cur], hd[cur], hn[cur ^ 1], hd[cur ^ 1]);
        cur ^= 1;
    }
    k_inv_spread<<<nrt, kThreads, 0, st>>>(a, r, hd[cur]);
    k_inv_walk2<<<nrt, kThreads, 0, st>>>(a, r, hist, d_T);  // no staging: every walk writes here
    cudaError_t e = cudaGetLastError();  // only this call's launches can have set it (peeked above)
    DevStatus hst{0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hst, dst, sizeof(hst), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return map_cuda_error(e);
    return hst.error;
}
