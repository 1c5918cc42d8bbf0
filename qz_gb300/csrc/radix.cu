// Segmented sorts of (32-bit key, 32-bit value) pairs in compact slot space
// for groups longer than a warp can sort (sm_103a, integer only).
//
//   * groups of up to kOT slots: one CTA sorts the whole group in shared
//     memory (8-bit LSD passes, digits constant across the group skipped),
//     reading and writing global memory once;
//   * longer groups: one LSD pass per launch over tiles of 2048, 4096 or
//     8192 slots ("onesweep").  Pass 0 takes the low 8..11 bits, passes 1..3
//     8 bits each, so keys of up to 27 bits (the rank keys of every round
//     after the first) sort in three passes.  One histogram kernel gives each
//     group's digit totals for all passes and marks the passes whose digit is
//     not constant in the group; the group runs only those.  Pass 0 needs no
//     stability (equal keys may leave in any order): tiles rank with shared
//     atomics and reserve their output with one atomic per digit on the
//     group's cursor; its tiles are fixed per CTA, so each CTA loads its next
//     tile by bulk copies (on an mbarrier) while it sorts the current one.
//     The later passes are stable: each tile takes a ticket in order, ranks
//     its digits per warp (a match on the digit's high four bits and ballots
//     on the low four), publishes its digit counts, and looks back over the
//     tiles before it in the same group for its exclusive prefix (decoupled
//     look-back), then scatters through shared memory so that each digit's run
//     leaves as coalesced writes.  A stable tile loads its keys to registers
//     and its values to shared memory (4-byte cp.async) together, and finds
//     its group through the tile table the histogram kernel writes.
//
// Look-back waits are bounded: a tile only waits on tiles that took earlier
// tickets, which publish their counts before they wait themselves; a wait that
// exceeds its iteration limit records QZGPU_TIMEOUT in the status word and the
// tile goes on (its positions stay inside its group), and the kernels whose
// stores such a failure could misplace return at entry once the status word
// is set; the host reads it after every round.  A bulk-copy wait that runs out
// records QZGPU_TIMEOUT too, and its tile stores nothing.
#include "engine.h"
#include "radix.cuh"
#include "scan.cuh"

namespace qz {

constexpr int kOItems = kOT / kThreads;   // 16 slots per thread
constexpr unsigned long long kFlagAgg = 1ull << 32;
constexpr unsigned long long kFlagInc = 2ull << 32;
constexpr unsigned kSpinLimit = 1u << 24;
constexpr unsigned kBulkSpinLimit = 1u << 22;  // mbarrier polls for a bulk copy (each may suspend for a while)

// Pass-0 bins at most (an 11-bit first digit) and digit-count words per
// listed group of the large-group sort (pass 0's bins, then 256 per later pass).
constexpr int kH0 = 2048;            // pass-0 bins at most (11 bits)
constexpr int kH4 = kH0 + 3 * 256;   // digit-count words per group

// ------------------------------------------------------------------ one-tile groups

// One CTA per group of kTileMin..kOT slots, every pass in shared memory
// (ping-pong key/value buffers).  The digit layout is the large-group sort's:
// pass 0 takes the low w0 bits (8..11) and needs no stability, so it ranks
// with shared-memory atomics over 2^w0 bins (the per-warp counter array
// doubles as them); passes 1..3 are stable 8-bit passes with warp
// match-based ranks.  Each warp takes an equal contiguous share of the group
// (a multiple of 32 slots), and digits that are equal across the whole group
// are skipped.  The group is read from (skey, sval) and written to (key, val)
// at the same slots; the two may be the same arrays.
__global__ void __launch_bounds__(kThreads) k_tile_sort(const int2* __restrict__ list, const int* __restrict__ d_count,
                                                        const uint32_t* skey, const int* sval, uint32_t* key,
                                                        int* val, int w0) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* k0 = reinterpret_cast<uint32_t*>(smem);
    int* v0 = reinterpret_cast<int*>(k0 + kOT);
    uint32_t* k1 = reinterpret_cast<uint32_t*>(v0 + kOT);
    int* v1 = reinterpret_cast<int*>(k1 + kOT);
    uint32_t(*wcnt)[256] = reinterpret_cast<uint32_t(*)[256]>(v1 + kOT);
    __shared__ uint32_t dig_off[256];
    __shared__ uint32_t sh[kWarps + 1];
    __shared__ uint32_t s_or[kWarps], s_and[kWarps];
    const unsigned w = warp_id(), ln = lane_id();
    const unsigned lt_mask = (1u << ln) - 1u;
    int cnt = *d_count;
    for (int g = blockIdx.x; g < cnt; g += gridDim.x) {
        int2 d = list[g];
        int s = d.x, len = d.y;
        uint32_t kor = 0, kand = 0xffffffffu;
        for (int i = threadIdx.x; i < len; i += kThreads) {
            uint32_t k = skey[s + i];
            k0[i] = k;
            v0[i] = sval[s + i];
            kor |= k;
            kand &= k;
        }
#pragma unroll
        for (int dd = 16; dd > 0; dd >>= 1) {
            kor |= __shfl_xor_sync(0xffffffffu, kor, dd);
            kand &= __shfl_xor_sync(0xffffffffu, kand, dd);
        }
        if (ln == 0) {
            s_or[w] = kor;
            s_and[w] = kand;
        }
        __syncthreads();
        kor = 0;
        kand = 0xffffffffu;
#pragma unroll
        for (int q = 0; q < kWarps; ++q) {
            kor |= s_or[q];
            kand &= s_and[q];
        }
        const uint32_t diff = kor ^ kand;
        const int nit = (len + kThreads - 1) / kThreads;  // slots per lane
        const int span = nit * 32;                         // slots per warp
        uint32_t* ks = k0;
        int* vs = v0;
        uint32_t* kd = k1;
        int* vd = v1;
        const uint32_t m0 = (1u << w0) - 1u;
        if (diff & m0) {
            // pass 0: unstable, shared atomics over 2^w0 bins
            uint32_t* bins = &wcnt[0][0];
            const int nbins = 1 << w0, per = nbins / kThreads;
            for (int i = threadIdx.x; i < nbins; i += kThreads) bins[i] = 0;
            __syncthreads();
            uint32_t rk[kOItems];
#pragma unroll
            for (int it = 0; it < kOItems; ++it) {
                const int i = (int)w * span + it * 32 + (int)ln;
                if (it < nit && i < len) rk[it] = atomicAdd(&bins[ks[i] & m0], 1u);
            }
            __syncthreads();
            {
                // this thread's run of `per` consecutive bins
                uint32_t c[kH0 / kThreads];
                uint32_t sum = 0;
#pragma unroll
                for (int q = 0; q < kH0 / kThreads; ++q) {
                    c[q] = q < per ? bins[threadIdx.x * per + q] : 0u;
                    sum += c[q];
                }
                uint32_t tot;
                uint32_t off = block_excl_sum(sum, sh, &tot);
#pragma unroll
                for (int q = 0; q < kH0 / kThreads; ++q) {
                    if (q < per) {
                        bins[threadIdx.x * per + q] = off;
                        off += c[q];
                    }
                }
            }
            __syncthreads();
#pragma unroll
            for (int it = 0; it < kOItems; ++it) {
                const int i = (int)w * span + it * 32 + (int)ln;
                if (it < nit && i < len) {
                    const uint32_t kv = ks[i];
                    const uint32_t p = bins[kv & m0] + rk[it];
                    kd[p] = kv;
                    vd[p] = vs[i];
                }
            }
            __syncthreads();
            uint32_t* tk = ks;
            ks = kd;
            kd = tk;
            int* tv = vs;
            vs = vd;
            vd = tv;
        }
        for (int pass = 1; pass < 4; ++pass) {
            const int shift = w0 + 8 * (pass - 1);
            if (((diff >> shift) & 255u) == 0) continue;
#pragma unroll
            for (int q = 0; q < kWarps; ++q) wcnt[q][threadIdx.x] = 0;
            __syncthreads();
            uint32_t rk[kOItems];
#pragma unroll
            for (int it = 0; it < kOItems; ++it) {
                if (it < nit) {
                    int i = (int)w * span + it * 32 + (int)ln;
                    bool valid = i < len;
                    unsigned dg = valid ? (ks[i] >> shift) & 255u : 256u;
                    unsigned peers = __match_any_sync(0xffffffffu, dg);
                    unsigned before = __popc(peers & lt_mask);
                    uint32_t prev = valid ? wcnt[w][dg] : 0u;
                    __syncwarp();
                    if (valid && before == 0) wcnt[w][dg] = prev + __popc(peers);
                    __syncwarp();
                    rk[it] = prev + before;
                }
            }
            __syncthreads();
            {
                unsigned dg = threadIdx.x;
                uint32_t run = 0;
#pragma unroll
                for (int q = 0; q < kWarps; ++q) {
                    uint32_t c = wcnt[q][dg];
                    wcnt[q][dg] = run;
                    run += c;
                }
                uint32_t tot;
                dig_off[dg] = block_excl_sum(run, sh, &tot);
            }
            __syncthreads();
#pragma unroll
            for (int it = 0; it < kOItems; ++it) {
                int i = (int)w * span + it * 32 + (int)ln;
                if (it < nit && i < len) {
                    uint32_t kv = ks[i];
                    unsigned dg = (kv >> shift) & 255u;
                    uint32_t p = dig_off[dg] + wcnt[w][dg] + rk[it];
                    kd[p] = kv;
                    vd[p] = vs[i];
                }
            }
            __syncthreads();
            uint32_t* tk = ks;
            ks = kd;
            kd = tk;
            int* tv = vs;
            vs = vd;
            vd = tv;
        }
        for (int i = threadIdx.x; i < len; i += kThreads) {
            key[s + i] = ks[i];
            val[s + i] = vs[i];
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ multi-tile groups
//
// Digit layout of one large-group sort: pass 0 takes the low w0 bits (8..11)
// and is unstable, so its ranking needs only shared-memory counters; passes
// 1..3 take 8 bits each above it.  Keys of at most w0 + 16 bits (the rank keys
// of a 25 MiB block need 26) therefore sort in three passes.  Per group the
// digit counts sit in kH4 words: pass 0's 2^w0 counts, then 256 per later pass.
// The look-back tile holds TILE slots (2048, 4096 or 8192; a tuning knob).

__device__ __forceinline__ int digit_shift(int pass, int w0) { return pass == 0 ? 0 : w0 + 8 * (pass - 1); }
__device__ __forceinline__ int h4_row(int pass) { return pass == 0 ? 0 : kH0 + 256 * (pass - 1); }

__global__ void __launch_bounds__(kThreads) k_big_prep(const int2* __restrict__ list, const int* __restrict__ d_count,
                                                       uint32_t* __restrict__ tcount, uint32_t* __restrict__ lens,
                                                       uint32_t* __restrict__ gmask, int tile) {
    int cnt = *d_count;
    for (int i = blockIdx.x * kThreads + threadIdx.x; i < cnt; i += gridDim.x * kThreads) {
        int len = list[i].y;
        tcount[i] = (uint32_t)((len + tile - 1) / tile);
        lens[i] = (uint32_t)len;
        gmask[i] = 0;
    }
}

// One CTA plans the large-group sort when the list is short (every launch of
// it counts): tiles and workspace offsets per group (exclusive scans of the
// tile counts and lengths), the total tile count, and cleared pass masks.
constexpr int kPlanMaxGroups = 32768;

constexpr int kPlanThreads = 1024;

__global__ void __launch_bounds__(kPlanThreads) k_big_plan(const int2* __restrict__ list,
                                                           const int* __restrict__ d_count,
                                                           uint32_t* __restrict__ tbase, uint32_t* __restrict__ wbase,
                                                           uint32_t* __restrict__ gmask,
                                                           int* __restrict__ total_tiles, int tile) {
    __shared__ uint32_t sht[kPlanThreads / 32 + 1], shw[kPlanThreads / 32 + 1];
    const int cnt = *d_count;
    // each thread owns a contiguous run of groups: its loads are issued
    // together, then one scan over the block
    const int per = (cnt + kPlanThreads - 1) / kPlanThreads;
    const int i0 = min(cnt, (int)threadIdx.x * per), i1 = min(cnt, i0 + per);
    uint32_t st = 0, sw = 0;
#pragma unroll 8
    for (int i = i0; i < i1; ++i) {
        const uint32_t len = (uint32_t)__ldg(&list[i].y);
        st += (len + tile - 1) / tile;
        sw += len;
    }
    const unsigned ln = lane_id(), wp = warp_id();
    const uint32_t it = warp_incl_sum(st), iw = warp_incl_sum(sw);
    if (ln == 31) {
        sht[wp] = it;
        shw[wp] = iw;
    }
    __syncthreads();
    if (wp == 0) {
        const uint32_t t = sht[ln], w = shw[ln];
        const uint32_t ti = warp_incl_sum(t), wi = warp_incl_sum(w);
        sht[ln] = ti - t;
        shw[ln] = wi - w;
        if (ln == 31) *total_tiles = (int)ti;
    }
    __syncthreads();
    uint32_t et = sht[wp] + it - st, ew = shw[wp] + iw - sw;
#pragma unroll 8
    for (int i = i0; i < i1; ++i) {
        const uint32_t len = (uint32_t)__ldg(&list[i].y);
        tbase[i] = et;
        wbase[i] = ew;
        gmask[i] = 0;
        et += (len + tile - 1) / tile;
        ew += len;
    }
}

// largest s in [0, n) with tbase[s] <= tau
__device__ __forceinline__ int big_seg_of_tile(const uint32_t* __restrict__ tbase, int n, uint32_t tau) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (tbase[mid] <= tau) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Digit counts of all passes per group (order-independent), by tile.
template <int TILE>
__global__ void __launch_bounds__(kThreads) k_big_hist(BigArgs a, const uint32_t* __restrict__ key,
                                                       uint32_t* __restrict__ h4, int w0) {
    constexpr int IT = TILE / kThreads;
    __shared__ uint32_t h0[kH0];
    __shared__ uint32_t h[3][256];
    __shared__ int s_seg;
    const int nb0 = 1 << w0;
    const uint32_t m0 = (uint32_t)nb0 - 1u;
    int TT = *a.ntiles, nseg = *a.nseg;
    for (int tau = blockIdx.x; tau < TT; tau += gridDim.x) {
        if (threadIdx.x == 0) {
            s_seg = big_seg_of_tile(a.tbase, nseg, (uint32_t)tau);
            a.tseg[tau] = (uint32_t)s_seg;  // the passes read it in one load
        }
        for (int i = threadIdx.x; i < nb0; i += kThreads) h0[i] = 0;
#pragma unroll
        for (int p = 0; p < 3; ++p) h[p][threadIdx.x] = 0;
        __syncthreads();
        int s = s_seg;
        int2 d = a.list[s];
        int j = tau - (int)a.tbase[s];
        int base = d.x + j * TILE;
        int cnt = min(TILE, d.y - j * TILE);
        uint32_t kr[IT];
        auto count = [&](uint32_t k) {
            atomicAdd(&h0[k & m0], 1u);
#pragma unroll
            for (int p = 0; p < 3; ++p) atomicAdd(&h[p][(k >> (w0 + 8 * p)) & 255u], 1u);
        };
        if (cnt == TILE) {  // full tile: no per-slot predicates
#pragma unroll
            for (int it = 0; it < IT; ++it) kr[it] = __ldg(key + base + it * kThreads + threadIdx.x);
#pragma unroll
            for (int it = 0; it < IT; ++it) count(kr[it]);
        } else {
#pragma unroll
            for (int it = 0; it < IT; ++it) {
                int i = it * kThreads + threadIdx.x;
                kr[it] = i < cnt ? __ldg(key + base + i) : 0u;
            }
#pragma unroll
            for (int it = 0; it < IT; ++it)
                if (it * kThreads + (int)threadIdx.x < cnt) count(kr[it]);
        }
        __syncthreads();
        uint32_t* g = h4 + (size_t)s * kH4;
        for (int i = threadIdx.x; i < nb0; i += kThreads) {
            uint32_t v = h0[i];
            if (v) atomicAdd(&g[i], v);
        }
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            uint32_t v = h[p][threadIdx.x];
            if (v) atomicAdd(&g[kH0 + 256 * p + threadIdx.x], v);
        }
        __syncthreads();
    }
}

// Zeroes the digit counts of the listed groups (their number read on the device).
__global__ void __launch_bounds__(kThreads) k_big_clear(uint4* __restrict__ h4, const int* __restrict__ d_count) {
    const long long n = (long long)*d_count * (kH4 / 4);
    for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < n; i += (long long)gridDim.x * kThreads)
        h4[i] = make_uint4(0, 0, 0, 0);
}

// Per group and pass: exclusive prefix over the pass's digits (in place), and
// the pass is marked needed unless one digit holds the whole group.
__global__ void __launch_bounds__(kThreads) k_big_bases(BigArgs a, uint32_t* __restrict__ h4, int w0) {
    __shared__ uint32_t sh[kWarps + 1];
    const int n = *a.nseg * 4;
    const int per0 = (1 << w0) / kThreads;  // pass-0 digits per thread (1..8)
    for (int r = blockIdx.x; r < n; r += gridDim.x) {
        const int s = r >> 2, p = r & 3;
        const uint32_t len = (uint32_t)a.list[s].y;
        uint32_t* row = h4 + (size_t)s * kH4 + h4_row(p);
        const int per = p == 0 ? per0 : 1;
        uint32_t v[kH0 / kThreads];
        uint32_t sum = 0;
        bool whole = false;
#pragma unroll
        for (int i = 0; i < kH0 / kThreads; ++i) {
            v[i] = i < per ? row[threadIdx.x * per + i] : 0u;
            sum += v[i];
            whole |= v[i] == len;
        }
        whole = __syncthreads_or(whole);
        uint32_t tot;
        uint32_t ex = block_excl_sum(sum, sh, &tot);
#pragma unroll
        for (int i = 0; i < kH0 / kThreads; ++i) {
            if (i < per) {
                row[threadIdx.x * per + i] = ex;
                ex += v[i];
            }
        }
        if (threadIdx.x == 0 && !whole) atomicOr(&a.gmask[s], 1u << p);
    }
}

// Passes a group runs: those whose digit is not constant, plus one trivial
// pass when that leaves a single one, so that no pass reads and writes the
// compact arrays at once.  The added pass leaves the order that matters: pass
// 0 (unstable) before a stable pass on the only varying digit, or the stable
// pass 1 after an only pass 0.
__device__ __forceinline__ uint32_t big_passes(uint32_t m) {
    return __popc(m) == 1 ? (m | (m == 1u ? 2u : 1u)) : m;
}

// Buffers of group s for pass p (a needed pass of its mask m).
struct BigRoute {
    const uint32_t* sk;
    const int* sv;
    uint32_t* dk;
    int* dv;
};

__device__ __forceinline__ BigRoute big_route(const BigBuffers& bb, const int2 d, uint32_t wb, uint32_t m, int p) {
    const int k = __popc(m & ((1u << p) - 1u));  // needed passes before this one
    const bool last = (m >> (p + 1)) == 0;
    // selects, not indexing, so the parameter arrays stay in registers
    const bool sodd = ((k - 1) & 1) != 0, dodd = (k & 1) != 0;
    BigRoute r;
    r.sk = k == 0 ? bb.key + d.x : (sodd ? bb.wsk[1] : bb.wsk[0]) + wb;
    r.sv = k == 0 ? bb.val + d.x : (sodd ? bb.wsv[1] : bb.wsv[0]) + wb;
    r.dk = last ? bb.key + d.x : (dodd ? bb.wsk[1] : bb.wsk[0]) + wb;
    r.dv = last ? bb.val + d.x : (dodd ? bb.wsv[1] : bb.wsv[0]) + wb;
    return r;
}

// Resident CTAs per SM each tile size is compiled for (registers per thread
// follow): 8192-slot tiles fit two by shared memory, 2048-slot tiles four.
template <int TILE>
constexpr int big_min_ctas() { return TILE >= 8192 ? 2 : (TILE <= 2048 ? 4 : 3); }

// Pass 0 (the low w0 bits).  Equal keys may leave a group sort in any order
// (the split gives them one rank), so this pass needs no stability: a tile
// ranks its slots with shared-memory atomics and reserves each digit's output
// range with one atomic on the group's digit cursor (its pass-0 base row), so
// it neither matches nor looks back.
template <int TILE>
__global__ void __launch_bounds__(kThreads, big_min_ctas<TILE>()) k_big_pass0(BigArgs a, uint32_t* __restrict__ h4,
                                                                              BigBuffers bb, int w0) {
    constexpr int IT = TILE / kThreads, WSPAN = TILE / kWarps;
    __shared__ uint32_t skey[TILE];
    __shared__ int sval[TILE];
    __shared__ int vst[TILE];  // the tile's values in slot order (asynchronous copies)
    __shared__ uint32_t cnt[kH0];
    __shared__ uint32_t gb[kH0];
    __shared__ uint32_t sh[kWarps + 1];
    __shared__ int s_seg;
    const unsigned w = warp_id(), ln = lane_id();
    const int nb0 = 1 << w0, per = nb0 / kThreads;
    const uint32_t m0 = (uint32_t)nb0 - 1u;
    const int TT = *a.ntiles;
    for (int tau = blockIdx.x; tau < TT; tau += gridDim.x) {
        if (threadIdx.x == 0) s_seg = (int)a.tseg[tau];
        for (int i = threadIdx.x; i < nb0; i += kThreads) cnt[i] = 0;
        __syncthreads();
        const int s = s_seg;
        const uint32_t m = big_passes(a.gmask[s]);
        const int2 d = a.list[s];
        const int j = tau - (int)a.tbase[s];
        const uint32_t wb = a.wbase[s];
        // the stable passes find everything about this tile in one place
        if (threadIdx.x == 0) {
            a.tdesc[tau] = make_int4(s, (int)m, d.x, (int)wb);
            a.tdesc2[tau] = make_int2(j, d.y);
        }
        if (!(m & 1u)) {
            __syncthreads();
            continue;  // uniform across the CTA
        }
        const BigRoute rt = big_route(bb, d, wb, m, 0);
        const uint32_t* sk = rt.sk;
        const int* sv = rt.sv;
        uint32_t* dk = rt.dk;
        int* dv = rt.dv;
        const int src = j * TILE;
        const int n = min(TILE, d.y - j * TILE);
        uint32_t kr[IT], rk[IT];
        // keys to registers and values to shared memory, all in flight at
        // once, then the ranking; full tiles without per-slot predicates
        if (n == TILE) {
#pragma unroll
            for (int it = 0; it < IT; ++it) {
                int i = (int)w * WSPAN + it * 32 + (int)ln;
                kr[it] = __ldcs(sk + src + i);
                cp_async4(vst + i, sv + src + i);
            }
#pragma unroll
            for (int it = 0; it < IT; ++it) rk[it] = atomicAdd(&cnt[kr[it] & m0], 1u);
        } else {
#pragma unroll
            for (int it = 0; it < IT; ++it) {
                int i = (int)w * WSPAN + it * 32 + (int)ln;
                kr[it] = i < n ? __ldcs(sk + src + i) : 0u;
                if (i < n) cp_async4(vst + i, sv + src + i);
            }
#pragma unroll
            for (int it = 0; it < IT; ++it) {
                int i = (int)w * WSPAN + it * 32 + (int)ln;
                rk[it] = i < n ? atomicAdd(&cnt[kr[it] & m0], 1u) : 0u;
            }
        }
        __syncthreads();
        {
            // this thread's run of `per` consecutive digits: tile offsets and
            // the group's output cursor for each
            uint32_t c[kH0 / kThreads];
            uint32_t sum = 0;
#pragma unroll
            for (int i = 0; i < kH0 / kThreads; ++i) {
                c[i] = i < per ? cnt[threadIdx.x * per + i] : 0u;
                sum += c[i];
            }
            uint32_t tot;
            uint32_t off = block_excl_sum(sum, sh, &tot);
#pragma unroll
            for (int i = 0; i < kH0 / kThreads; ++i) {
                if (i < per) {
                    const int dg = threadIdx.x * per + i;
                    const uint32_t base = c[i] ? atomicAdd(&h4[(size_t)s * kH4 + dg], c[i]) : 0u;
                    cnt[dg] = off;
                    gb[dg] = base - off;
                    off += c[i];
                }
            }
        }
        cp_async_wait_all();  // each thread reads back only the values it copied
        __syncthreads();
#pragma unroll
        for (int it = 0; it < IT; ++it) {
            int i = (int)w * WSPAN + it * 32 + (int)ln;
            if (i < n) {
                uint32_t lp = cnt[kr[it] & m0] + rk[it];
                skey[lp] = kr[it];
                sval[lp] = vst[i];
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += kThreads) {
            uint32_t kv = skey[i];
            uint32_t dst = gb[kv & m0] + (uint32_t)i;
            dk[dst] = kv;
            dv[dst] = sval[i];
        }
        __syncthreads();
    }
}

// Pass 0 with bulk copies, double-buffered.  A CTA's tiles are fixed (tau,
// tau + grid, ...), so thread 0 issues the next tile's copies before the CTA
// ranks and scatters the current one: the next tile's keys and values are in
// flight during the whole of the current tile.  Each run is copied as its
// 16-byte-aligned cover (one bulk copy for the keys, one for the values,
// completed on the buffer's mbarrier; the arrays are 256-byte aligned and
// followed by other arrays of the same allocation, so the cover stays inside
// it) and indexed from its offset in the buffer.  Once a tile's keys and
// values are in registers, its buffer doubles as the scatter staging.
struct P0Desc {
    int s, m;  // group, pass mask
    int2 d;    // group's first slot and length
    int j, wb; // tile within the group, workspace base
    int n;     // slots in this tile
    int ok, ov;  // element offsets of the keys and of the values in their buffers
    int load;  // copies issued (the group runs pass 0)
};

template <int TILE>
constexpr int p0_buf() { return TILE + 8; }  // a 4-byte run of TILE slots rounded out to 16 bytes
template <int TILE>
constexpr size_t p0_bulk_smem() { return sizeof(uint32_t) * (4 * (size_t)p0_buf<TILE>() + 2 * kH0); }
template <int TILE>
constexpr int p0_bulk_ctas() { return TILE >= 8192 ? 1 : (TILE <= 2048 ? 4 : 2); }

template <int TILE>
__global__ void __launch_bounds__(kThreads, p0_bulk_ctas<TILE>()) k_big_pass0_bulk(BigArgs a,
                                                                                 uint32_t* __restrict__ h4,
                                                                                 BigBuffers bb, int w0,
                                                                                 DevStatus* st) {
    constexpr int IT = TILE / kThreads, WSPAN = TILE / kWarps, BUF = p0_buf<TILE>();
    extern __shared__ __align__(128) uint32_t p0smem[];
    uint32_t* kb = p0smem;                          // [2][BUF] keys
    int* vb = reinterpret_cast<int*>(p0smem + 2 * BUF);  // [2][BUF] values
    uint32_t* cnt = p0smem + 4 * BUF;               // [kH0] per-digit counts, then tile offsets
    uint32_t* gb = cnt + kH0;                       // [kH0] group cursor minus tile offset
    __shared__ uint32_t sh[kWarps + 1];
    __shared__ __align__(8) unsigned long long bar[2];
    __shared__ P0Desc sd[2];
    const unsigned w = warp_id(), ln = lane_id();
    const int nb0 = 1 << w0, per = nb0 / kThreads;
    const uint32_t m0 = (uint32_t)nb0 - 1u;
    const int TT = *a.ntiles;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init_fence();
    }
    __syncthreads();
    // thread 0: tile tau's descriptor (written out for the stable passes too)
    // and, when its group runs pass 0, its copies into buffer bi
    auto issue = [&](int tau, int bi) {
        P0Desc D;
        D.s = (int)a.tseg[tau];
        D.m = (int)big_passes(a.gmask[D.s]);
        D.d = a.list[D.s];
        D.j = tau - (int)a.tbase[D.s];
        D.wb = (int)a.wbase[D.s];
        D.n = min(TILE, D.d.y - D.j * TILE);
        a.tdesc[tau] = make_int4(D.s, D.m, D.d.x, D.wb);
        a.tdesc2[tau] = make_int2(D.j, D.d.y);
        D.load = D.m & 1;
        D.ok = D.ov = 0;
        if (D.load) {
            const BigRoute rt = big_route(bb, D.d, (uint32_t)D.wb, (uint32_t)D.m, 0);
            const uint32_t* ks = rt.sk + (size_t)D.j * TILE;
            const int* vs = rt.sv + (size_t)D.j * TILE;
            D.ok = (int)(((uintptr_t)ks & 15u) >> 2);
            D.ov = (int)(((uintptr_t)vs & 15u) >> 2);
            const unsigned kbytes = ((unsigned)(D.ok + D.n) * 4u + 15u) & ~15u;
            const unsigned vbytes = ((unsigned)(D.ov + D.n) * 4u + 15u) & ~15u;
            fence_proxy_async_smem();  // the buffer's last reads and writes come first
            mbar_arrive_expect_tx(&bar[bi], kbytes + vbytes);
            bulk_g2s(kb + bi * BUF, reinterpret_cast<const void*>((uintptr_t)ks & ~(uintptr_t)15), kbytes, &bar[bi]);
            bulk_g2s(vb + bi * BUF, reinterpret_cast<const void*>((uintptr_t)vs & ~(uintptr_t)15), vbytes, &bar[bi]);
        }
        sd[bi] = D;
    };
    if (threadIdx.x == 0 && (int)blockIdx.x < TT) issue((int)blockIdx.x, 0);
    unsigned par = 0;  // bit bi: parity of buffer bi's next phase
    int b = 0;
    for (int tau = blockIdx.x; tau < TT; tau += gridDim.x, b ^= 1) {
        if (threadIdx.x == 0 && tau + (int)gridDim.x < TT) issue(tau + (int)gridDim.x, b ^ 1);
        for (int i = threadIdx.x; i < nb0; i += kThreads) cnt[i] = 0;
        __syncthreads();  // sd[b] (issued one tile earlier) and the cleared counts
        const P0Desc D = sd[b];
        if (!D.load) {
            __syncthreads();  // everyone has read sd[b] before it is issued again
            continue;
        }
        bool ok = mbar_wait(&bar[b], par >> b & 1u, kBulkSpinLimit);
        par ^= 1u << b;
        if (!ok) {
            // copies that never completed: record it, give them a second
            // bounded wait (they write this buffer) and store nothing
            if (threadIdx.x == 0) report(st, QZGPU_TIMEOUT, 22, tau);
            mbar_wait(&bar[b], (par >> b & 1u) ^ 1u, kBulkSpinLimit);
        }
        if (!__syncthreads_and(ok)) {
            __syncthreads();
            continue;
        }
        const BigRoute rt = big_route(bb, D.d, (uint32_t)D.wb, (uint32_t)D.m, 0);
        uint32_t* dk = rt.dk;
        int* dv = rt.dv;
        const int n = D.n;
        uint32_t* kc = kb + b * BUF;
        int* vc = vb + b * BUF;
        uint32_t kr[IT], rk[IT];
        int vr[IT];
        if (n == TILE) {
#pragma unroll
            for (int it = 0; it < IT; ++it) {
                const int i = (int)w * WSPAN + it * 32 + (int)ln;
                kr[it] = kc[D.ok + i];
                vr[it] = vc[D.ov + i];
            }
#pragma unroll
            for (int it = 0; it < IT; ++it) rk[it] = atomicAdd(&cnt[kr[it] & m0], 1u);
        } else {
#pragma unroll
            for (int it = 0; it < IT; ++it) {
                const int i = (int)w * WSPAN + it * 32 + (int)ln;
                kr[it] = i < n ? kc[D.ok + i] : 0u;
                vr[it] = i < n ? vc[D.ov + i] : 0;
                rk[it] = i < n ? atomicAdd(&cnt[kr[it] & m0], 1u) : 0u;
            }
        }
        __syncthreads();
        {
            uint32_t c[kH0 / kThreads];
            uint32_t sum = 0;
#pragma unroll
            for (int i = 0; i < kH0 / kThreads; ++i) {
                c[i] = i < per ? cnt[threadIdx.x * per + i] : 0u;
                sum += c[i];
            }
            uint32_t tot;
            uint32_t off = block_excl_sum(sum, sh, &tot);
#pragma unroll
            for (int i = 0; i < kH0 / kThreads; ++i) {
                if (i < per) {
                    const int dg = threadIdx.x * per + i;
                    const uint32_t base = c[i] ? atomicAdd(&h4[(size_t)D.s * kH4 + dg], c[i]) : 0u;
                    cnt[dg] = off;
                    gb[dg] = base - off;
                    off += c[i];
                }
            }
        }
        __syncthreads();
        // the buffer's contents are in registers: stage the scatter there
#pragma unroll
        for (int it = 0; it < IT; ++it) {
            const int i = (int)w * WSPAN + it * 32 + (int)ln;
            if (i < n) {
                const uint32_t lp = cnt[kr[it] & m0] + rk[it];
                kc[lp] = kr[it];
                vc[lp] = vr[it];
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += kThreads) {
            const uint32_t kv = kc[i];
            const uint32_t dst = gb[kv & m0] + (uint32_t)i;
            dk[dst] = kv;
            dv[dst] = vc[i];
        }
        __syncthreads();  // the buffer and sd[b] are free for the tile after next
    }
}

// One stable 8-bit pass (1..3) with decoupled look-back.  RANK: how a warp
// finds the lanes with the same digit (warp_digit_peers).  EARLY: the tile's
// digit counts come first, from shared-memory atomics, and are published
// before the stable ranking, so that the tiles behind this one find them while
// it ranks (otherwise the counts are published after the ranking, which
// yields them as well).
template <int TILE, int RANK, bool EARLY>
__global__ void __launch_bounds__(kThreads, big_min_ctas<TILE>()) k_big_pass(
    BigArgs a, const uint32_t* __restrict__ h4, int pass, int w0, unsigned epoch, BigBuffers bb,
    unsigned long long* status, unsigned* ticket, DevStatus* st, unsigned spin_limit, int silent_tile) {
    constexpr int IT = TILE / kThreads, WSPAN = TILE / kWarps;
    __shared__ uint32_t skey[TILE];
    __shared__ int sval[TILE];
    __shared__ int vst[TILE];  // the tile's values in slot order (asynchronous copies)
    __shared__ uint32_t wcnt[kWarps][256];
    __shared__ uint32_t tcnt[EARLY ? 256 : 1];  // the tile's digit counts (early publication)
    __shared__ uint32_t dig_off[256];
    __shared__ uint32_t gbase[256];
    __shared__ uint32_t sh[kWarps + 1];
    __shared__ int s_tau;
    __shared__ int4 s_d;
    __shared__ int2 s_d2;
    const unsigned w = warp_id(), ln = lane_id();
    const int shift = digit_shift(pass, w0);
    const unsigned long long ep = (unsigned long long)epoch << 34;
    // an earlier pass that failed leaves keys whose digits no longer match the
    // group histograms, so the positions below would not stay in the group
    if (failed(st)) return;
    const int TT = *a.ntiles;
    for (;;) {
        if (threadIdx.x == 0) {
            // the ticket, then the tile's descriptor in one dependent load
            s_tau = (int)atomicAdd(ticket, 1u);
            if (s_tau < TT) {
                s_d = a.tdesc[s_tau];
                s_d2 = a.tdesc2[s_tau];
            }
        }
#pragma unroll
        for (int q = 0; q < kWarps; ++q) wcnt[q][threadIdx.x] = 0;
        if (EARLY) tcnt[threadIdx.x] = 0;
        __syncthreads();
        int tau = s_tau;
        if (tau >= TT) return;
        const int s = s_d.x;
        const uint32_t m = (uint32_t)s_d.y;
        if (!(m >> pass & 1u)) {
            // nothing to sort on this digit: the group's slots stay put and no
            // tile of it looks back at this one
            __syncthreads();
            continue;
        }
        const int2 d = make_int2(s_d.z, s_d2.y);
        const int j = s_d2.x;
        const BigRoute rt = big_route(bb, d, (uint32_t)s_d.w, m, pass);
        const uint32_t* srck = rt.sk;
        const int* srcv = rt.sv;
        uint32_t* dstk = rt.dk;
        int* dstv = rt.dv;
        int srcbase = j * TILE;
        int cnt = min(TILE, d.y - j * TILE);
        uint32_t rk[IT], kr[IT];
        // all of the tile's keys (to registers) and values (to shared memory)
        // in flight at once, then the ranking
#pragma unroll
        for (int it = 0; it < IT; ++it) {
            int i = (int)w * WSPAN + it * 32 + (int)ln;
            kr[it] = i < cnt ? __ldg(srck + srcbase + i) : 0u;
            if (i < cnt) cp_async4(vst + i, srcv + srcbase + i);
        }
        // this thread's digit: the group's base for it, fetched while the keys
        // are in flight; stored to shared memory only after the ranking, so
        // that the ranking starts as soon as the first keys arrive
        const uint32_t hb = h4[(size_t)s * kH4 + h4_row(pass) + threadIdx.x];
        volatile unsigned long long* my = status + (size_t)tau * 256 + threadIdx.x;
        const bool silent = j == silent_tile;  // failure-detection test only
        if (EARLY) {
            // counts only (no order): one shared atomic per slot
#pragma unroll
            for (int it = 0; it < IT; ++it) {
                int i = (int)w * WSPAN + it * 32 + (int)ln;
                if (i < cnt) atomicAdd(&tcnt[(kr[it] >> shift) & 255u], 1u);
            }
            __syncthreads();
            const uint32_t c = tcnt[threadIdx.x];
            if (j == 0)
                *my = ep | kFlagInc | c;
            else if (!silent)
                *my = ep | kFlagAgg | c;
        }
        // full tiles (all but a group's last) rank without per-slot
        // predicates.  The two loop bodies also keep the compiler from moving
        // key loads down into the ranking: measured 28.8 against 34.6 ms per
        // chunk forward on one lane, with long-scoreboard stalls halved.
        if (cnt == TILE) {
#pragma unroll
            for (int it = 0; it < IT; ++it) rk[it] = warp_digit_rank<RANK>((kr[it] >> shift) & 255u, true, wcnt[w]);
        } else {
#pragma unroll
            for (int it = 0; it < IT; ++it) {
                int i = (int)w * WSPAN + it * 32 + (int)ln;
                rk[it] = warp_digit_rank<RANK>((kr[it] >> shift) & 255u, i < cnt, wcnt[w]);
            }
        }
        gbase[threadIdx.x] = hb;
        __syncthreads();
        {
            unsigned dg = threadIdx.x;
            uint32_t run = 0;
#pragma unroll
            for (int q = 0; q < kWarps; ++q) {
                uint32_t c = wcnt[q][dg];
                wcnt[q][dg] = run;
                run += c;
            }
            // publish this tile's count (unless published early), then find
            // the counts of the tiles before it in the same group
            uint32_t excl = 0;
            if (j == 0) {
                if (!EARLY) *my = ep | kFlagInc | run;
            } else {
                if (!EARLY && !silent) *my = ep | kFlagAgg | run;
                int p = tau - 1;
                for (;;) {
                    volatile unsigned long long* q = status + (size_t)p * 256 + dg;
                    unsigned long long v = *q;
                    unsigned spins = 0;
                    while (((v >> 34) != epoch || (v & (3ull << 32)) == 0) && spins < spin_limit) {
                        __nanosleep(32);
                        v = *q;
                        ++spins;
                    }
                    if (spins >= spin_limit) {
                        report(st, QZGPU_TIMEOUT, 20, tau);
                        break;
                    }
                    excl += (uint32_t)(v & 0xffffffffull);
                    if (v & kFlagInc) break;
                    --p;
                }
                if (!silent) *my = ep | kFlagInc | (excl + run);
            }
            uint32_t tot;
            dig_off[dg] = block_excl_sum(run, sh, &tot);
            gbase[dg] += excl;
        }
        cp_async_wait_all();  // each thread reads back only the values it copied
        __syncthreads();
#pragma unroll
        for (int it = 0; it < IT; ++it) {
            int i = (int)w * WSPAN + it * 32 + (int)ln;
            if (i < cnt) {
                uint32_t kv = kr[it];
                unsigned dg = (kv >> shift) & 255u;
                uint32_t lp = dig_off[dg] + wcnt[w][dg] + rk[it];
                skey[lp] = kv;
                sval[lp] = vst[i];
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < cnt; i += kThreads) {
            uint32_t kv = skey[i];
            unsigned dg = (kv >> shift) & 255u;
            uint32_t dst = gbase[dg] + ((uint32_t)i - dig_off[dg]);
            dstk[dst] = kv;
            dstv[dst] = sval[i];
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ host side

namespace {
int grid_cap(long long work, int per_cta, int cap) {
    long long g = (work + per_cta - 1) / per_cta;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}
}  // namespace

size_t tile_sort_smem() { return (size_t)kOT * 16 + sizeof(uint32_t) * kWarps * 256; }
size_t big_hist_words() { return kH4; }

namespace {
// Width of pass 0's digit for keys of key_bits bits: wide enough that three
// 8-bit passes above it cover the key, up to the tuned maximum; 8 otherwise.
// (A wide first digit for keys that need four passes anyway was measured:
// with 2048 bins of a few slots each, pass 0's scatter leaves uncoalesced and
// its time doubled, 9.4 to 20.5 ms per chunk forward on one lane.)
int first_digit_bits(int key_bits, int max_bits) {
    if (key_bits > 24 && key_bits <= 16 + max_bits) return key_bits - 16;
    return 8;
}
}  // namespace

void sort_tile_groups(Storage* S, const int2* list, const int* d_count, int host_count, long long elems,
                      const uint32_t* skey, const int* sval, uint32_t* key, int* val, int key_bits,
                      cudaStream_t st) {
    if (host_count <= 0) return;
    const int w0 = first_digit_bits(key_bits, S->tune.first_digit_max);
    smem_limit_once<k_tile_sort>((int)tile_sort_smem(), S->device);
    QZ_LAUNCH(S, st, "k_tile_sort", 16 * elems,
              k_tile_sort<<<grid_cap(host_count, 1, S->sms * S->tune.tile_ctas_per_sm), kThreads, tile_sort_smem(),
                            st>>>(list, d_count, skey, sval, key, val, w0));
}

namespace {

// Tile bases (and the total tile count) per listed group, cleared digit masks.
void big_plan(Storage* S, const int2* list, const int* d_count, int host_count, int tile, cudaStream_t st) {
    FwdBuffers& f = S->f;
    int* cnt = S->counters;
    if (host_count <= kPlanMaxGroups) {
        QZ_LAUNCH(S, st, "k_big_plan", 20ll * host_count,
                  k_big_plan<<<1, kPlanThreads, 0, st>>>(list, d_count, f.ltbase, f.lwbase, f.gmask,
                                                         cnt + CNT_LTILES, tile));
    } else {
        QZ_LAUNCH(S, st, "k_big_prep", 20ll * host_count,
                  k_big_prep<<<grid_cap(host_count, kThreads, S->sms * 4), kThreads, 0, st>>>(list, d_count, f.ltc,
                                                                                             f.llen, f.gmask, tile));
        scan_exclusive(S, f.ltc, f.ltbase, 0, d_count, (uint32_t*)(cnt + CNT_LTILES), st);
        scan_exclusive(S, f.llen, f.lwbase, 0, d_count, nullptr, st);
    }
}

template <int TILE>
void big_sort_run(Storage* S, const BigArgs& a, const BigBuffers& bb, uint32_t* h4, int host_count,
                  long long elems, int w0, int npass, cudaStream_t st) {
    FwdBuffers& f = S->f;
    int* cnt = S->counters;
    const int sms = S->sms;
    const int grid = sms * 4;
    QZ_LAUNCH(S, st, "k_big_hist", 4 * elems, k_big_hist<TILE><<<grid, kThreads, 0, st>>>(a, bb.key, h4, w0));
    QZ_LAUNCH(S, st, "k_big_bases", 4ll * kH4 * host_count,
              k_big_bases<<<grid_cap(4ll * host_count, 1, sms * 8), kThreads, 0, st>>>(a, h4, w0));
    // pass 0: unstable, no look-back (bytes are an upper bound: passes whose
    // digit is constant in a group are skipped for that group)
    if (S->tune.pass0_bulk) {
        smem_limit_once<k_big_pass0_bulk<TILE>>((int)p0_bulk_smem<TILE>(), S->device);
        QZ_LAUNCH(S, st, "k_big_pass0", 16 * elems,
                  k_big_pass0_bulk<TILE><<<sms * p0_bulk_ctas<TILE>(), kThreads, p0_bulk_smem<TILE>(), st>>>(
                      a, h4, bb, w0, S->status));
    } else {
        QZ_LAUNCH(S, st, "k_big_pass0", 16 * elems, k_big_pass0<TILE><<<grid, kThreads, 0, st>>>(a, h4, bb, w0));
    }
    // stable passes: decoupled look-back over a persistent grid, tiles taken
    // by ticket (a tile waits only on tiles of earlier tickets, whose CTAs are
    // resident, so the grid may exceed what fits at once)
    const int pgrid = sms * S->tune.big_ctas_per_sm;
    for (int pass = 1; pass < npass; ++pass) {
        unsigned epoch = ++S->radix_epoch & 0x3fffffffu;
        if (epoch == 0) epoch = ++S->radix_epoch & 0x3fffffffu;
        unsigned* ticket = reinterpret_cast<unsigned*>(cnt + CNT_TICKET);
        if (!S->dry) cudaMemsetAsync(ticket, 0, sizeof(unsigned), st);
        const bool test = S->tune.lookback_test && pass == 1;
        const unsigned spin = test ? 4096u : kSpinLimit;
        const int silent = test ? 1 : -1;
#define QZ_BIG_PASS(R, E)                                                                                  \
    QZ_LAUNCH(S, st, "k_big_pass", 16 * elems,                                                             \
              (k_big_pass<TILE, R, E><<<pgrid, kThreads, 0, st>>>(a, h4, pass, w0, epoch, bb, f.status64, \
                                                                  ticket, S->status, spin, silent)))
        const bool early = S->tune.early_counts != 0;
        switch (S->tune.rank_mode * 2 + (early ? 1 : 0)) {
            case 2: QZ_BIG_PASS(1, false); break;
            case 3: QZ_BIG_PASS(1, true); break;
            case 4: QZ_BIG_PASS(2, false); break;
            case 5: QZ_BIG_PASS(2, true); break;
            case 1: QZ_BIG_PASS(0, true); break;
            default: QZ_BIG_PASS(0, false); break;
        }
#undef QZ_BIG_PASS
    }
}

}  // namespace

void sort_big_groups(Storage* S, const int2* list, const int* d_count, int host_count, long long elems,
                     uint32_t* key, int* val, int key_bits, cudaStream_t st) {
    if (host_count <= 0) return;
    FwdBuffers& f = S->f;
    int* cnt = S->counters;
    const int tile = S->tune.big_tile;
    big_plan(S, list, d_count, host_count, tile, st);
    BigArgs a{list, d_count, f.ltbase, f.lwbase, cnt + CNT_LTILES, f.gmask, f.tseg, f.tdesc, f.tdesc2};
    BigBuffers bb{key, val, {f.wsk[0], f.wsk[1]}, {f.wsv[0], f.wsv[1]}};
    uint32_t* h4 = f.h4;
    // digit counts of the listed groups cleared (host_count may be a bound)
    QZ_LAUNCH(S, st, "k_big_clear", 4ll * kH4 * host_count,
              k_big_clear<<<grid_cap(host_count * (long long)(kH4 / 4), kThreads, S->sms * 4), kThreads, 0, st>>>(
                  reinterpret_cast<uint4*>(h4), d_count));
    const int w0 = first_digit_bits(key_bits, S->tune.first_digit_max);
    const int npass = key_bits <= w0 + 16 ? 3 : 4;  // a fourth pass only when the key needs it
    switch (tile) {
        case 2048: big_sort_run<2048>(S, a, bb, h4, host_count, elems, w0, npass, st); break;
        case 8192: big_sort_run<8192>(S, a, bb, h4, host_count, elems, w0, npass, st); break;
        default: big_sort_run<4096>(S, a, bb, h4, host_count, elems, w0, npass, st); break;
    }
}

}  // namespace qz
