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
//   2. list ranking of the single LF cycle: rows r with r % stride == 0 are
//      rulers; each ruler walks LF to the next ruler (walk 1), ruler
//      distances to row 0 come from pointer jumping, and each ruler walks its
//      stretch again writing T[n - d] = F(row) (walk 2), F read from the
//      block's symbol start table in shared memory.
// Every row is read twice; every wait is a bounded loop and a broken LF cycle
// (corrupt input) is reported as QZGPU_DATA_CORRUPT.
#include <algorithm>
#include <mutex>

#include "engine.h"
#include "scan.cuh"

namespace qz {

constexpr int kIRItems = kInitTile / kThreads;  // 16
constexpr int kIRWarpSpan = kInitTile / kWarps;  // 512

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
    const unsigned lt_mask = (1u << ln) - 1u;
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
    // all of the tile's symbols in flight at once, then the ranking
#pragma unroll
    for (int it = 0; it < kIRItems; ++it) {
        int i = (int)w * kIRWarpSpan + it * 32 + (int)ln;
        cu[it] = i < cnt ? (unsigned)__ldg(a.U + s0 + i) : 256u;
    }
#pragma unroll
    for (int it = 0; it < kIRItems; ++it) {
        int i = (int)w * kIRWarpSpan + it * 32 + (int)ln;
        bool valid = i < cnt;
        unsigned c = cu[it];
        unsigned peers = __match_any_sync(0xffffffffu, c);
        unsigned before = __popc(peers & lt_mask);
        uint32_t prev = valid ? wcnt[w][c] : 0u;
        __syncwarp();
        if (valid && before == 0) wcnt[w][c] = prev + __popc(peers);
        __syncwarp();
        cc[it] = (uint8_t)c;
        rk[it] = prev + before;
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

struct RulerArgs {
    const int2* rtiles;  // (block, first local ruler) per CTA
    int* next0;
    int* dist0;
    int* len;
};

__global__ void __launch_bounds__(kThreads) k_inv_walk1(InvArgs a, RulerArgs r) {
    int2 rt = r.rtiles[blockIdx.x];
    int b = rt.x;
    int bs = a.off[b], n = a.off[b + 1] - bs;
    int mask = (1 << a.stride_log2) - 1;
    int M = (n >> a.stride_log2) + 1;
    int lq = rt.y + threadIdx.x;
    if (lq >= M) return;
    const int* LF = a.LF + bs + b;
    int q = a.rbase[b] + lq;
    int cur = lq << a.stride_log2;
    int steps = 0;
    bool ok = true;
    const unsigned long long pol = l2_keep_policy();
    do {
        cur = ld_keep(LF + cur, pol);
        ++steps;
        if (cur < 0 || cur > n || steps > n + 1) {
            ok = false;
            break;
        }
    } while (cur & mask);
    if (!ok) {
        report(a.st, QZGPU_DATA_CORRUPT, 10, b);
        r.next0[q] = -1;
        r.dist0[q] = 0;
        r.len[q] = 0;
        return;
    }
    int nl = cur >> a.stride_log2;
    r.next0[q] = nl == 0 ? -1 : a.rbase[b] + nl;
    r.dist0[q] = steps;
    r.len[q] = steps;
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

__global__ void __launch_bounds__(kThreads) k_inv_walk2(InvArgs a, RulerArgs r, const int* __restrict__ next,
                                                        const int* __restrict__ dist,
                                                        const uint32_t* __restrict__ hist,
                                                        uint8_t* __restrict__ T) {
    __shared__ int C[257];       // first row of each present symbol, then n + 1
    __shared__ uint8_t sym[256];  // the present symbols, ascending
    __shared__ int s_cnt[kWarps + 1];
    int2 rt = r.rtiles[blockIdx.x];
    int b = rt.x;
    int bs = a.off[b], n = a.off[b + 1] - bs;
    int m = (n + kInitTile - 1) / kInitTile;
    // symbol starts in the first column (1 + count of smaller symbols), kept
    // for the symbols that occur only, so the search below takes log2(sigma)
    // steps
    {
        const uint32_t* hb = hist + (size_t)256 * a.tbase[b];
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
    }
    __syncthreads();
    const int sigma = s_cnt[kWarps];
    int M = (n >> a.stride_log2) + 1;
    int lq = rt.y + threadIdx.x;
    if (lq >= M) return;
    const int* LF = a.LF + bs + b;
    int q = a.rbase[b] + lq;
    if (lq == 0 && (next[q] != -1 || dist[q] != n + 1)) {
        report(a.st, QZGPU_DATA_CORRUPT, 11, b);
        return;
    }
    int d = (n + 1) - dist[q];
    int cur = lq << a.stride_log2;
    int L = r.len[q];
    if (d < 0 || d > n) {
        report(a.st, QZGPU_DATA_CORRUPT, 12, b);
        return;
    }
    // The walk visits suffixes n-d, n-d-1, ...: a run of consecutive output
    // bytes written downwards.  Bytes are packed into 32-bit words aligned on
    // their absolute address, so the run leaves as word stores; a word not
    // completely filled by this walk is stored byte by byte.
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
            for (int q = 0; q < 4; ++q)
                if (have & (1u << q)) reinterpret_cast<uint8_t*>(word_at)[q] = (uint8_t)(word >> (8 * q));
        }
    };
    for (int t = 0; t < L; ++t) {
        // the next row is loaded first; the symbol search below overlaps it
        const int nxt = ld_keep(LF + cur, pol);
        int s = n - d;
        if (s < 0) {
            report(a.st, QZGPU_DATA_CORRUPT, 13, b);
            return;
        }
        if (s < n) {
            int lo = 0, hi = sigma - 1;
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (C[mid] <= cur) lo = mid; else hi = mid - 1;
            }
            lo = sym[lo];
            uintptr_t addr = reinterpret_cast<uintptr_t>(out + s);
            uintptr_t wa = addr & ~(uintptr_t)3;
            if (wa != word_at) {
                flush();
                word_at = wa;
                word = 0;
                have = 0;
            }
            int q = (int)(addr & 3);
            word |= (uint32_t)lo << (8 * q);
            have |= 1u << q;
        }
        cur = nxt;
        ++d;
    }
    flush();
}

int inverse_run(Storage* S, int nb, const int* n, const int* idx, const uint8_t* d_U, uint8_t* d_T,
                cudaStream_t st) {
    if (nb < 0 || nb > S->cap_blocks) return QZGPU_BAD_PARAMETER;
    long long N = 0;
    for (int b = 0; b < nb; ++b) {
        if (n[b] < 0) return QZGPU_BAD_PARAMETER;
        if (n[b] > 0 && (idx[b] < 1 || idx[b] > n[b])) return QZGPU_DATA_CORRUPT;
        N += n[b];
    }
    if (N > S->cap_bytes) return QZGPU_BAD_PARAMETER;
    S->stats = qzgpu_stats{};
    S->launches = 0;
    if (N == 0) return QZGPU_NO_ERROR;
    const int stride_log2 = S->tune.ruler_log2;  // rulers every 2^stride_log2 rows
    const int stride = 1 << stride_log2;

    std::vector<int> off(nb + 1, 0), tbase(nb + 1, 0), rbase(nb + 1, 0);
    std::vector<int2> tiles, rtiles;
    int maxM = 1;
    for (int b = 0; b < nb; ++b) {
        off[b + 1] = off[b] + n[b];
        int m = (n[b] + kInitTile - 1) / kInitTile;
        tbase[b + 1] = tbase[b] + m;
        for (int s = off[b]; s < off[b + 1]; s += kInitTile) tiles.push_back(make_int2(b, s));
        int M = n[b] > 0 ? n[b] / stride + 1 : 0;
        rbase[b + 1] = rbase[b] + M;
        for (int q = 0; q < M; q += kThreads) rtiles.push_back(make_int2(b, q));
        if (M > maxM) maxM = M;
    }
    int Mtot = rbase[nb];
    if ((size_t)tbase[nb] * 256 > S->hist_cap) return QZGPU_BAD_PARAMETER;
    size_t need = sizeof(int) * (4 * (nb + 1)) + sizeof(int2) * (tiles.size() + rtiles.size()) + 256;
    if (need > S->pin_tab_bytes) return QZGPU_BAD_PARAMETER;
    char* p = S->pin_tab;
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
    h2d(S->tiles, h_tiles, sizeof(int2) * tiles.size());
    h2d(v.rtiles, h_rt, sizeof(int2) * rtiles.size());
    if (e == cudaSuccess) e = cudaMemsetAsync(S->status, 0, sizeof(DevStatus), st);
    if (e != cudaSuccess) return map_cuda_error(e);

    InvArgs a{d_U, S->blk_off, S->blk_idx, S->blk_tbase, S->blk_aux_off, S->tiles, v.LF, stride_log2, S->status};
    int ntiles = (int)tiles.size();
    int hist_len = tbase[nb] * 256;
    long long rows = N + nb;
    // U read once for the histogram, once for the ranks; LF written once
    QZ_LAUNCH(S, st, "k_inv_up", N, k_inv_up<<<ntiles, kThreads, 0, st>>>(a, S->hist));
    scan_exclusive(S, S->hist, S->hist, hist_len, nullptr, nullptr, st);
    QZ_LAUNCH(S, st, "k_inv_down", 5 * N, k_inv_down<<<ntiles, kThreads, 0, st>>>(a, S->hist));
    RulerArgs r{v.rtiles, v.rnext[0], v.rdist[0], v.rlen};
    int nrt = (int)rtiles.size();
    // every row's LF entry read once; 12 bytes per ruler written
    QZ_LAUNCH(S, st, "k_inv_walk1", 4 * rows + 12ll * Mtot, k_inv_walk1<<<nrt, kThreads, 0, st>>>(a, r));
    int cur = 0;
    int jgrid = (int)std::min<long long>(((long long)Mtot + kThreads - 1) / kThreads, (long long)S->sms * 16);
    for (long long span = 1; span < maxM + 1; span <<= 1) {
        QZ_LAUNCH(S, st, "k_inv_jump", 24ll * Mtot,
                  k_inv_jump<<<jgrid, kThreads, 0, st>>>(Mtot, v.rnext[cur], v.rdist[cur], v.rnext[cur ^ 1],
                                                          v.rdist[cur ^ 1]));
        cur ^= 1;
    }
    // every row's LF entry read again and one output byte written per row
    QZ_LAUNCH(S, st, "k_inv_walk2", 4 * rows + N + 12ll * Mtot,
              k_inv_walk2<<<nrt, kThreads, 0, st>>>(a, r, v.rnext[cur], v.rdist[cur], S->hist, d_T));
    DevStatus* hst = reinterpret_cast<DevStatus*>(S->pin_rd);
    e = cudaMemcpyAsync(hst, S->status, sizeof(DevStatus), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return map_cuda_error(e);
    prof_flush(S);
    if (hst->error) {
        if (debug_on()) debug_log("device status %d at %d detail %lld", hst->error, hst->where, hst->detail);
        return hst->error;
    }
    S->stats.kernel_launches = S->launches;
    S->stats.alg_bytes = 12 * N;
    return QZGPU_NO_ERROR;
}

}  // namespace qz

// ------------------------------------------------------------------ allocation-free inverse
//
// For callers that cannot allocate device memory while they run: a pipeline
// stage inside a host runtime that owns every device allocation up front
// (and forbids cudaMalloc/cudaFree later), or code on a thread that must not
// take the allocator's locks.  The caller passes device input and output;
// all scratch of the inverse lives in one file-scope array below, sized for
// blocks of up to QZGPU_NOALLOC_MAX_BLOCK bytes.

namespace qz {
namespace noalloc {

constexpr long long kMaxN = QZGPU_NOALLOC_MAX_BLOCK;
constexpr long long kMaxTiles = (kMaxN + kInitTile - 1) / kInitTile;
constexpr int kStrideLog2 = 5;
constexpr long long kMaxRulers = (kMaxN >> kStrideLog2) + 1;
constexpr long long kMaxRTiles = (kMaxRulers + kThreads - 1) / kThreads;

constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }
// byte offsets inside the scratch array
constexpr size_t kOffLF = 0;
constexpr size_t kOffHist = align256(kOffLF + 4 * (kMaxN + 2));
constexpr size_t kOffPartial = align256(kOffHist + 4 * 256 * kMaxTiles);
constexpr size_t kOffRuler = align256(kOffPartial + 4 * 1024);
constexpr size_t kRulerBytes = align256(4 * kMaxRulers);
constexpr size_t kOffTiles = kOffRuler + 5 * kRulerBytes;
constexpr size_t kOffRTiles = align256(kOffTiles + 8 * kMaxTiles);
constexpr size_t kOffTables = align256(kOffRTiles + 8 * kMaxRTiles);  // off, idx, tbase, rbase
constexpr size_t kOffStatus = align256(kOffTables + 4 * 16);
constexpr size_t kBytes = align256(kOffStatus + sizeof(DevStatus));
static_assert(kBytes <= (6u << 20), "allocation-free scratch exceeds its stated 6 MiB");

}  // namespace noalloc

// Every GPU that loads this library holds this array until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[noalloc::kBytes];

// Per-block tables of a single-block inverse, built on the device.
__global__ void k_noalloc_tables(char* scratch, int n, int index) {
    using namespace noalloc;
    int* tab = reinterpret_cast<int*>(scratch + kOffTables);
    int m = (n + kInitTile - 1) / kInitTile;
    int M = (n >> kStrideLog2) + 1;
    if (threadIdx.x == 0) {
        tab[0] = 0;  // off
        tab[1] = n;
        tab[2] = index;  // idx
        tab[4] = 0;      // tbase
        tab[5] = m;
        tab[6] = 0;      // rbase
        tab[7] = M;
        *reinterpret_cast<DevStatus*>(scratch + kOffStatus) = DevStatus{0, 0, 0};
    }
    int2* tiles = reinterpret_cast<int2*>(scratch + kOffTiles);
    for (int j = threadIdx.x; j < m; j += blockDim.x) tiles[j] = make_int2(0, j * kInitTile);
    int2* rtiles = reinterpret_cast<int2*>(scratch + kOffRTiles);
    int nrt = (M + kThreads - 1) / kThreads;
    for (int j = threadIdx.x; j < nrt; j += blockDim.x) rtiles[j] = make_int2(0, j * kThreads);
}

namespace {

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[256];

// Device address of the scratch array for the current device, looked up once
// per device (host code must not use the array's name as a device address).
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
    char* sc = nullptr;
    int rc = noalloc_scratch(&sc);
    if (rc) return rc;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    int* tab = reinterpret_cast<int*>(sc + kOffTables);
    int m = (n + kInitTile - 1) / kInitTile;
    int M = (n >> kStrideLog2) + 1;
    int nrt = (M + kThreads - 1) / kThreads;
    int* rul = reinterpret_cast<int*>(sc + kOffRuler);
    int* rnext0 = rul;
    int* rdist0 = reinterpret_cast<int*>(sc + kOffRuler + kRulerBytes);
    int* rnext1 = reinterpret_cast<int*>(sc + kOffRuler + 2 * kRulerBytes);
    int* rdist1 = reinterpret_cast<int*>(sc + kOffRuler + 3 * kRulerBytes);
    int* rlen = reinterpret_cast<int*>(sc + kOffRuler + 4 * kRulerBytes);
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
    RulerArgs r{reinterpret_cast<const int2*>(sc + kOffRTiles), rnext0, rdist0, rlen};
    k_inv_walk1<<<nrt, kThreads, 0, st>>>(a, r);
    int* nx[2] = {rnext0, rnext1};
    int* ds[2] = {rdist0, rdist1};
    int cur = 0;
    int jgrid = (M + kThreads - 1) / kThreads;
    for (long long span = 1; span < (long long)M + 1; span <<= 1) {
        k_inv_jump<<<jgrid, kThreads, 0, st>>>(M, nx[cur], ds[cur], nx[cur ^ 1], ds[cur ^ 1]);
        cur ^= 1;
    }
    k_inv_walk2<<<nrt, kThreads, 0, st>>>(a, r, nx[cur], ds[cur], hist, d_T);
    cudaError_t e = cudaGetLastError();
    DevStatus hst{0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hst, dst, sizeof(hst), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return map_cuda_error(e);
    return hst.error;
}
