// Forward BWT of a batch of blocks by prefix doubling on sm_103a.
//
// Replaces the suffix sort that libbsc runs inside bsc_compress for
// blockSorter = BWT (reached from crates/qz-lib/src/compression/bsc.rs:172-183;
// libbsc's bwt.cpp / libsais are not in the reference tree).
//
// Layout in HBM: all blocks of a batch are concatenated; block b owns text
// positions and suffix-array positions [off[b], off[b+1]).  Suffixes of
// different blocks are never compared: the first sort is segmented by block
// and a suffix that runs past its block end gets an end key.
//
// Phases:
//   1. per-block byte histogram -> dense symbol codes, sigma_b, and the number
//      K_b of symbols that fit a 32-bit key in base sigma_b;
//   2. initial keys: K_b symbols per suffix, padded with the smallest code;
//   3. sort each block's suffixes by key (segment classes below), then split
//      into groups of equal key: group rank = SA position of the group head;
//   4. rounds h = K_b, 2K_b, 4K_b, ...: for every suffix x still in a group,
//      key = R[x+h] + h + 1 if x+h is inside the block, else (n_b - i), which
//      orders a suffix that ends first before any longer one; sort inside
//      each group, split, repeat until every group is a singleton;
//   5. extract U and the primary index (libsais convention).
//
// Groups are kept in a compact work list in SA order (slot arrays P = SA
// position, W = suffix, G = group head).  Per round each group is sorted by
// the kernel of its size class: <= 16 in registers, <= 4096 in shared memory,
// larger ones by a segmented LSD radix sort (8-bit digits, warp match-based
// stable ranking, shared-memory staged scatter).
#include "engine.h"
#include "scan.cuh"

namespace qz {

constexpr int kSplitItems = 8;
constexpr int kSplitTile = kThreads * kSplitItems;
constexpr int kRItems = kRT / kThreads;  // 16 elements per thread in a radix tile
constexpr int kRWarpSpan = kRT / kWarps; // 512 contiguous elements per warp

// ------------------------------------------------------------------ per-block alphabet

__global__ void __launch_bounds__(kThreads) k_block_hist(const uint8_t* __restrict__ T,
                                                         const int2* __restrict__ tiles,
                                                         const int* __restrict__ off,
                                                         uint32_t* __restrict__ bhist) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    int2 tl = tiles[blockIdx.x];
    int b = tl.x, s0 = tl.y;
    int end = min(off[b + 1], s0 + kInitTile);
    for (int base = s0; base < end; base += kThreads) {
        int x = base + threadIdx.x;
        unsigned c = x < end ? (unsigned)T[x] : 256u;
        unsigned peers = __match_any_sync(0xffffffffu, c);
        if (c < 256u && lane_id() == (unsigned)(__ffs(peers) - 1)) atomicAdd(&h[c], __popc(peers));
    }
    __syncthreads();
    uint32_t v = h[threadIdx.x];
    if (v) atomicAdd(&bhist[(size_t)b * 256 + threadIdx.x], v);
}

__global__ void __launch_bounds__(kThreads) k_block_alpha(const uint32_t* __restrict__ bhist,
                                                          uint8_t* __restrict__ code, int* __restrict__ Kout,
                                                          int* __restrict__ sigma_out) {
    __shared__ uint32_t sh[kWarps + 1];
    int b = blockIdx.x;
    uint32_t present = bhist[(size_t)b * 256 + threadIdx.x] ? 1u : 0u;
    uint32_t tot;
    uint32_t ex = block_excl_sum(present, sh, &tot);
    code[(size_t)b * 256 + threadIdx.x] = (uint8_t)ex;
    if (threadIdx.x == 0) {
        int K;
        if (tot <= 1) {
            K = 1 << 30;  // one symbol: every suffix is a prefix of a longer one
        } else {
            unsigned long long v = 1;
            K = 0;
            while (v * tot <= (1ull << 32)) {
                v *= tot;
                ++K;
            }
        }
        Kout[b] = K;
        sigma_out[b] = (int)tot;
    }
}

// Initial keys: K_b symbols in base sigma_b (at most 32 symbols since sigma_b >= 2).
__global__ void __launch_bounds__(kThreads) k_init_keys(const uint8_t* __restrict__ T,
                                                        const int2* __restrict__ tiles,
                                                        const int* __restrict__ off,
                                                        const uint8_t* __restrict__ code,
                                                        const int* __restrict__ Kb,
                                                        const int* __restrict__ sigb,
                                                        uint32_t* __restrict__ key, int* __restrict__ W,
                                                        int* __restrict__ G) {
    __shared__ uint8_t scode[256];
    __shared__ uint8_t stext[kInitTile + 64];
    int2 tl = tiles[blockIdx.x];
    int b = tl.x, s0 = tl.y;
    int bstart = off[b], bend = off[b + 1];
    int K = Kb[b], sigma = sigb[b];
    scode[threadIdx.x] = code[(size_t)b * 256 + threadIdx.x];
    int Kc = sigma > 1 ? K : 0;
    int wend = min(bend, s0 + kInitTile + Kc);
    for (int x = s0 + threadIdx.x; x < wend; x += kThreads) stext[x - s0] = T[x];
    __syncthreads();
    int end = min(bend, s0 + kInitTile);
    for (int x = s0 + threadIdx.x; x < end; x += kThreads) {
        unsigned long long k = 0;
        for (int d = 0; d < Kc; ++d) {
            int y = x + d;
            unsigned c = y < bend ? scode[stext[y - s0]] : 0u;
            k = k * (unsigned)sigma + c;
        }
        key[x] = (uint32_t)k;
        W[x] = x;
        G[x] = bstart;
    }
}

// ------------------------------------------------------------------ group sorts

__device__ __forceinline__ unsigned long long pack_kv(uint32_t k, int v) {
    return ((unsigned long long)k << 32) | (uint32_t)v;
}

__global__ void __launch_bounds__(kThreads) k_sort_small(const int2* __restrict__ list,
                                                         const int* __restrict__ d_count,
                                                         uint32_t* __restrict__ key, int* __restrict__ W) {
    int cnt = *d_count;
    for (int i = blockIdx.x * kThreads + threadIdx.x; i < cnt; i += gridDim.x * kThreads) {
        int2 d = list[i];
        int s = d.x, len = d.y;
        if (len == 2) {
            uint32_t k0 = key[s], k1 = key[s + 1];
            if (k1 < k0) {
                int w0 = W[s], w1 = W[s + 1];
                key[s] = k1;
                key[s + 1] = k0;
                W[s] = w1;
                W[s + 1] = w0;
            }
            continue;
        }
        unsigned long long v[kSmallMax];
#pragma unroll
        for (int j = 0; j < kSmallMax; ++j) v[j] = j < len ? pack_kv(key[s + j], W[s + j]) : ~0ull;
#pragma unroll
        for (int k = 2; k <= kSmallMax; k <<= 1) {
#pragma unroll
            for (int jj = k >> 1; jj > 0; jj >>= 1) {
#pragma unroll
                for (int a = 0; a < kSmallMax; ++a) {
                    int l = a ^ jj;
                    if (l > a) {
                        bool up = (a & k) == 0;
                        unsigned long long x = v[a], y = v[l];
                        bool sw = up ? (x > y) : (x < y);
                        v[a] = sw ? y : x;
                        v[l] = sw ? x : y;
                    }
                }
            }
        }
#pragma unroll
        for (int j = 0; j < kSmallMax; ++j) {
            if (j < len) {
                key[s + j] = (uint32_t)(v[j] >> 32);
                W[s + j] = (int)(uint32_t)v[j];
            }
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_sort_medium(const int2* __restrict__ list,
                                                          const int* __restrict__ d_count,
                                                          uint32_t* __restrict__ key, int* __restrict__ W) {
    __shared__ unsigned long long buf[kMedMax];
    int cnt = *d_count;
    for (int i = blockIdx.x; i < cnt; i += gridDim.x) {
        int2 d = list[i];
        int s = d.x, len = d.y;
        int np = 2;
        while (np < len) np <<= 1;
        for (int j = threadIdx.x; j < np; j += kThreads) buf[j] = j < len ? pack_kv(key[s + j], W[s + j]) : ~0ull;
        __syncthreads();
        for (int k = 2; k <= np; k <<= 1) {
            for (int jj = k >> 1; jj > 0; jj >>= 1) {
                for (int a = threadIdx.x; a < np; a += kThreads) {
                    int l = a ^ jj;
                    if (l > a) {
                        unsigned long long x = buf[a], y = buf[l];
                        bool up = (a & k) == 0;
                        if (up ? (x > y) : (x < y)) {
                            buf[a] = y;
                            buf[l] = x;
                        }
                    }
                }
                __syncthreads();
            }
        }
        for (int j = threadIdx.x; j < len; j += kThreads) {
            key[s + j] = (uint32_t)(buf[j] >> 32);
            W[s + j] = (int)(uint32_t)buf[j];
        }
        __syncthreads();
    }
}

// Large groups: tiles per group and workspace layout (groups back to back).
__global__ void __launch_bounds__(kThreads) k_large_prep(const int2* __restrict__ list,
                                                         const int* __restrict__ d_count,
                                                         uint32_t* __restrict__ tcount,
                                                         uint32_t* __restrict__ lens) {
    int cnt = *d_count;
    for (int i = blockIdx.x * kThreads + threadIdx.x; i < cnt; i += gridDim.x * kThreads) {
        int len = list[i].y;
        tcount[i] = (uint32_t)((len + kRT - 1) / kRT);
        lens[i] = (uint32_t)len;
    }
}

// largest s in [0, n) with tbase[s] <= tau
__device__ __forceinline__ int seg_of_tile(const uint32_t* __restrict__ tbase, int n, uint32_t tau) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (tbase[mid] <= tau) lo = mid; else hi = mid - 1;
    }
    return lo;
}

struct LargeArgs {
    const int2* list;
    const int* nseg;
    const uint32_t* tbase;
    const uint32_t* wbase;
    const int* ntiles;
    int* hist_len;  // written: 256 * tiles
};

__global__ void __launch_bounds__(kThreads) k_large_up(LargeArgs a, const uint32_t* __restrict__ srck,
                                                       int src_compact, int shift,
                                                       uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[256];
    __shared__ int s_seg;
    int TT = *a.ntiles, nseg = *a.nseg;
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.hist_len = 256 * TT;
    for (int tau = blockIdx.x; tau < TT; tau += gridDim.x) {
        if (threadIdx.x == 0) s_seg = seg_of_tile(a.tbase, nseg, (uint32_t)tau);
        h[threadIdx.x] = 0;
        __syncthreads();
        int s = s_seg;
        int2 d = a.list[s];
        int j = tau - (int)a.tbase[s];
        int m = (d.y + kRT - 1) / kRT;
        int base = (src_compact ? d.x : (int)a.wbase[s]) + j * kRT;
        int cnt = min(kRT, d.y - j * kRT);
        for (int q = 0; q < kRT; q += kThreads) {
            int i = q + threadIdx.x;
            unsigned dg = i < cnt ? (srck[base + i] >> shift) & 255u : 256u;
            unsigned peers = __match_any_sync(0xffffffffu, dg);
            if (dg < 256u && lane_id() == (unsigned)(__ffs(peers) - 1)) atomicAdd(&h[dg], __popc(peers));
        }
        __syncthreads();
        hist[(size_t)256 * a.tbase[s] + (size_t)threadIdx.x * m + j] = h[threadIdx.x];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kThreads) k_large_down(LargeArgs a, const uint32_t* __restrict__ hist,
                                                         const uint32_t* __restrict__ srck,
                                                         const int* __restrict__ srcv, int src_compact,
                                                         uint32_t* __restrict__ dstk, int* __restrict__ dstv,
                                                         int dst_compact, int shift) {
    __shared__ uint32_t skey[kRT];
    __shared__ int sval[kRT];
    __shared__ uint32_t wcnt[kWarps][256];
    __shared__ uint32_t dig_off[256];
    __shared__ uint32_t gbase[256];
    __shared__ uint32_t sh[kWarps + 1];
    __shared__ int s_seg;
    int TT = *a.ntiles, nseg = *a.nseg;
    const unsigned w = warp_id(), ln = lane_id();
    const unsigned lt_mask = (1u << ln) - 1u;
    for (int tau = blockIdx.x; tau < TT; tau += gridDim.x) {
        if (threadIdx.x == 0) s_seg = seg_of_tile(a.tbase, nseg, (uint32_t)tau);
#pragma unroll
        for (int q = 0; q < kWarps; ++q) wcnt[q][threadIdx.x] = 0;
        __syncthreads();
        int s = s_seg;
        int2 d = a.list[s];
        int j = tau - (int)a.tbase[s];
        int m = (d.y + kRT - 1) / kRT;
        int srcbase = (src_compact ? d.x : (int)a.wbase[s]) + j * kRT;
        int cnt = min(kRT, d.y - j * kRT);
        uint32_t kk[kRItems];
        int vv[kRItems];
        uint32_t rk[kRItems];
#pragma unroll
        for (int it = 0; it < kRItems; ++it) {
            int i = (int)w * kRWarpSpan + it * 32 + (int)ln;
            bool valid = i < cnt;
            uint32_t kv = valid ? srck[srcbase + i] : 0u;
            int vl = valid ? srcv[srcbase + i] : 0;
            unsigned dg = valid ? (kv >> shift) & 255u : 256u;
            unsigned peers = __match_any_sync(0xffffffffu, dg);
            unsigned before = __popc(peers & lt_mask);
            uint32_t prev = valid ? wcnt[w][dg] : 0u;
            __syncwarp();
            if (valid && before == 0) wcnt[w][dg] = prev + __popc(peers);
            __syncwarp();
            kk[it] = kv;
            vv[it] = vl;
            rk[it] = prev + before;
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
            uint32_t ex = block_excl_sum(run, sh, &tot);
            dig_off[dg] = ex;
            int dstbase = dst_compact ? d.x : (int)a.wbase[s];
            gbase[dg] = hist[(size_t)256 * a.tbase[s] + (size_t)dg * m + j] - a.wbase[s] + (uint32_t)dstbase;
        }
        __syncthreads();
#pragma unroll
        for (int it = 0; it < kRItems; ++it) {
            int i = (int)w * kRWarpSpan + it * 32 + (int)ln;
            if (i < cnt) {
                unsigned dg = (kk[it] >> shift) & 255u;
                uint32_t lp = dig_off[dg] + wcnt[w][dg] + rk[it];
                skey[lp] = kk[it];
                sval[lp] = vv[it];
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

// ------------------------------------------------------------------ split into groups

struct SplitArgs {
    const int* A;      // active slots of this split
    int* A_next;       // receives the survivor count
    const uint32_t* key;
    const int* G;
    const int* P;  // null: slot k is SA position k (first split)
    const int* W;
    int* R;
    int* SA;
    int* Pn;
    int* Wn;
    int* Gn;
    int2* list0;
    int2* list1;
    int2* list2;
    int* counters;
    int* part_surv;  // [kSplitGrid]
    int* part_head;  // [kSplitGrid]
};

struct SplitItems {
    uint32_t k[kSplitItems];
    int g[kSplitItems];
    bool head[kSplitItems];
    bool nhead[kSplitItems];
};

// Loads this thread's kSplitItems consecutive slots starting at k0 (< hi) and
// computes group-head flags for each and for its successor.
__device__ __forceinline__ void split_load(const SplitArgs& a, int A, int k0, int hi, SplitItems& it) {
    if (k0 + kSplitItems <= hi) {
        const uint4* kp = reinterpret_cast<const uint4*>(a.key + k0);
        const int4* gp = reinterpret_cast<const int4*>(a.G + k0);
        uint4 k01 = kp[0], k23 = kp[1];
        int4 g01 = gp[0], g23 = gp[1];
        it.k[0] = k01.x; it.k[1] = k01.y; it.k[2] = k01.z; it.k[3] = k01.w;
        it.k[4] = k23.x; it.k[5] = k23.y; it.k[6] = k23.z; it.k[7] = k23.w;
        it.g[0] = g01.x; it.g[1] = g01.y; it.g[2] = g01.z; it.g[3] = g01.w;
        it.g[4] = g23.x; it.g[5] = g23.y; it.g[6] = g23.z; it.g[7] = g23.w;
    } else {
#pragma unroll
        for (int i = 0; i < kSplitItems; ++i) {
            int k = k0 + i;
            it.k[i] = k < hi ? a.key[k] : 0u;
            it.g[i] = k < hi ? a.G[k] : 0;
        }
    }
    uint32_t pk = 0;
    int pg = 0;
    if (k0 > 0) {
        pk = a.key[k0 - 1];
        pg = a.G[k0 - 1];
    }
#pragma unroll
    for (int i = 0; i < kSplitItems; ++i) {
        int k = k0 + i;
        if (k == 0) it.head[i] = true;
        else if (i == 0) it.head[i] = it.g[0] != pg || it.k[0] != pk;
        else it.head[i] = it.g[i] != it.g[i - 1] || it.k[i] != it.k[i - 1];
    }
#pragma unroll
    for (int i = 0; i < kSplitItems; ++i) {
        int k = k0 + i;
        if (k >= hi) {
            it.nhead[i] = true;
        } else if (k + 1 >= A) {
            it.nhead[i] = true;
        } else if (i + 1 < kSplitItems && k + 1 < hi) {
            it.nhead[i] = it.head[i + 1];
        } else {
            it.nhead[i] = a.G[k + 1] != it.g[i] || a.key[k + 1] != it.k[i];
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_split_count(SplitArgs a) {
    __shared__ uint32_t shs[kWarps + 1];
    __shared__ int shm[kWarps + 1];
    int A = *a.A;
    int lo, hi;
    chunk_range(A, gridDim.x, blockIdx.x, kSplitTile, &lo, &hi);
    uint32_t surv = 0;
    int lasthead = -1;
    for (int base = lo; base < hi; base += kSplitTile) {
        int k0 = base + threadIdx.x * kSplitItems;
        if (k0 < hi) {
            SplitItems it;
            split_load(a, A, k0, hi, it);
#pragma unroll
            for (int i = 0; i < kSplitItems; ++i) {
                int k = k0 + i;
                if (k < hi) {
                    surv += (it.head[i] && it.nhead[i]) ? 0u : 1u;
                    if (it.head[i]) lasthead = k;
                }
            }
        }
    }
    uint32_t tot;
    block_excl_sum(surv, shs, &tot);
    int mx;
    block_incl_max(lasthead, shm, &mx);
    if (threadIdx.x == 0) {
        a.part_surv[blockIdx.x] = (int)tot;
        a.part_head[blockIdx.x] = mx;
    }
}

// One CTA: exclusive sum of survivors and exclusive max of group heads over
// the split chunks; new active count; resets the descriptor counters.
__global__ void __launch_bounds__(kThreads) k_split_top(SplitArgs a) {
    __shared__ uint32_t shs[kWarps + 1];
    __shared__ int shm[kWarps + 1];
    uint32_t carry = 0;
    int mcarry = -1;
    for (int base = 0; base < kSplitGrid; base += kThreads) {
        int i = base + threadIdx.x;
        uint32_t v = (uint32_t)a.part_surv[i];
        int h = a.part_head[i];
        uint32_t tot;
        uint32_t ex = block_excl_sum(v, shs, &tot);
        int mtot;
        int inc = block_incl_max(h, shm, &mtot);
        int exm = __shfl_up_sync(0xffffffffu, inc, 1);
        __shared__ int lastw[kWarps];
        if (lane_id() == 31) lastw[warp_id()] = inc;
        __syncthreads();
        if (lane_id() == 0) exm = warp_id() == 0 ? -1 : lastw[warp_id() - 1];
        __syncthreads();
        a.part_surv[i] = (int)(carry + ex);
        a.part_head[i] = max(mcarry, exm);
        carry += tot;
        mcarry = max(mcarry, mtot);
    }
    if (threadIdx.x == 0) {
        *a.A_next = (int)carry;
        a.counters[CNT_SMALL] = 0;
        a.counters[CNT_MED] = 0;
        a.counters[CNT_LARGE] = 0;
    }
}

__device__ __forceinline__ int block_excl_max(int v, int* sh, int* total) {
    int inc = block_incl_max(v, sh, total);
    __shared__ int lastw[kWarps];
    int ex = __shfl_up_sync(0xffffffffu, inc, 1);
    if (lane_id() == 31) lastw[warp_id()] = inc;
    __syncthreads();
    if (lane_id() == 0) ex = warp_id() == 0 ? INT32_MIN : lastw[warp_id() - 1];
    __syncthreads();
    return ex;
}

__global__ void __launch_bounds__(kThreads) k_split_apply(SplitArgs a) {
    __shared__ uint32_t shs[kWarps + 1];
    __shared__ int shm[kWarps + 1];
    __shared__ unsigned long long shl[kWarps + 1];
    __shared__ int lbase[3];
    int A = *a.A;
    int lo, hi;
    chunk_range(A, gridDim.x, blockIdx.x, kSplitTile, &lo, &hi);
    uint32_t surv_carry = (uint32_t)a.part_surv[blockIdx.x];
    int head_carry = a.part_head[blockIdx.x];
    for (int base = lo; base < hi; base += kSplitTile) {
        int k0 = base + threadIdx.x * kSplitItems;
        SplitItems it;
        bool any = k0 < hi;
        if (any) split_load(a, A, k0, hi, it);
        uint32_t mysurv = 0;
        int myhead = -1;
        if (any) {
#pragma unroll
            for (int i = 0; i < kSplitItems; ++i) {
                int k = k0 + i;
                if (k < hi) {
                    mysurv += (it.head[i] && it.nhead[i]) ? 0u : 1u;
                    if (it.head[i]) myhead = k;
                }
            }
        }
        uint32_t stot;
        uint32_t sex = block_excl_sum(mysurv, shs, &stot);
        int mtot;
        int hex = block_excl_max(myhead, shm, &mtot);
        int kg = max(head_carry, hex);
        uint32_t dest = surv_carry + sex;
        // group heads and class counts of group tails
        int kgs[kSplitItems];
        unsigned long long cls_cnt = 0;
        if (any) {
#pragma unroll
            for (int i = 0; i < kSplitItems; ++i) {
                int k = k0 + i;
                if (k < hi) {
                    if (it.head[i]) kg = k;
                    kgs[i] = kg;
                    bool single = it.head[i] && it.nhead[i];
                    if (!single && it.nhead[i]) {
                        int L = k - kg + 1;
                        int c = L <= kSmallMax ? 0 : (L <= kMedMax ? 1 : 2);
                        cls_cnt += 1ull << (16 * c);
                    }
                }
            }
        }
        unsigned long long ctot;
        unsigned long long cex = block_excl_sum(cls_cnt, shl, &ctot);
        if (threadIdx.x == 0) {
            lbase[0] = (ctot & 0xffff) ? atomicAdd(&a.counters[CNT_SMALL], (int)(ctot & 0xffff)) : 0;
            lbase[1] = ((ctot >> 16) & 0xffff) ? atomicAdd(&a.counters[CNT_MED], (int)((ctot >> 16) & 0xffff)) : 0;
            lbase[2] = ((ctot >> 32) & 0xffff) ? atomicAdd(&a.counters[CNT_LARGE], (int)((ctot >> 32) & 0xffff)) : 0;
        }
        __syncthreads();
        if (any) {
            int lp[3] = {lbase[0] + (int)(cex & 0xffff), lbase[1] + (int)((cex >> 16) & 0xffff),
                         lbase[2] + (int)((cex >> 32) & 0xffff)};
            int2* lists[3] = {a.list0, a.list1, a.list2};
#pragma unroll
            for (int i = 0; i < kSplitItems; ++i) {
                int k = k0 + i;
                if (k < hi) {
                    int kgi = kgs[i];
                    int rank = a.P ? a.P[kgi] : kgi;
                    int w = a.W[k];
                    int pk = a.P ? a.P[k] : k;
                    a.R[w] = rank;
                    bool single = it.head[i] && it.nhead[i];
                    if (single) {
                        a.SA[pk] = w;
                    } else {
                        a.Pn[dest] = pk;
                        a.Wn[dest] = w;
                        a.Gn[dest] = rank;
                        if (it.nhead[i]) {
                            int L = k - kgi + 1;
                            int c = L <= kSmallMax ? 0 : (L <= kMedMax ? 1 : 2);
                            lists[c][lp[c]++] = make_int2((int)dest - L + 1, L);
                        }
                        ++dest;
                    }
                }
            }
        }
        // carry to the next tile of this chunk
        surv_carry += stot;
        head_carry = max(head_carry, mtot);
        __syncthreads();
    }
}

// ------------------------------------------------------------------ rounds

__global__ void __launch_bounds__(kThreads) k_gather(const int* __restrict__ d_A, const int* __restrict__ W,
                                                     const int* __restrict__ R, const int* __restrict__ off,
                                                     int nb, const int* __restrict__ Kb, int round,
                                                     uint32_t* __restrict__ key) {
    int A = *d_A;
    for (int k = blockIdx.x * kThreads + threadIdx.x; k < A; k += gridDim.x * kThreads) {
        int x = W[k];
        int b = block_of(off, nb, x);
        int bs = __ldg(off + b), n = __ldg(off + b + 1) - bs;
        long long h = round >= 31 ? (long long)n : ((long long)__ldg(Kb + b) << round);
        if (h > n) h = n;
        int i = x - bs;
        uint32_t kv;
        if ((long long)i + h < n) kv = (uint32_t)R[x + (int)h] + (uint32_t)h + 1u;
        else kv = (uint32_t)(n - i);
        key[k] = kv;
    }
}

__global__ void __launch_bounds__(kThreads) k_extract(int N, const int* __restrict__ SA, const int* __restrict__ R,
                                                      const uint8_t* __restrict__ T, const int* __restrict__ off,
                                                      int nb, uint8_t* __restrict__ U, int* __restrict__ idx,
                                                      const int* __restrict__ aux_rate,
                                                      const int* __restrict__ aux_off, int* __restrict__ aux,
                                                      DevStatus* st) {
    for (int j = blockIdx.x * kThreads + threadIdx.x; j < N; j += gridDim.x * kThreads) {
        int b = block_of(off, nb, j);
        int bs = __ldg(off + b), n = __ldg(off + b + 1) - bs;
        int jl = j - bs;
        int s = SA[j] - bs;
        if (s < 0 || s >= n) {
            report(st, QZGPU_GPU_ERROR, 1, j);
            continue;
        }
        int p = R[bs] - bs + 1;
        if (jl == 0) U[bs] = T[bs + n - 1];
        if (s == 0) {
            idx[b] = p;
        } else {
            int u = (jl + 1 < p) ? jl + 1 : jl;
            U[bs + u] = T[bs + s - 1];
        }
        if (aux_rate) {
            int r = aux_rate[b];
            if (r > 0 && s > 0 && (s & (r - 1)) == 0) aux[aux_off[b] + s / r - 1] = jl + 1;
        }
    }
}

// ------------------------------------------------------------------ host driver

namespace {

struct Launch {
    cudaStream_t st;
    int sms;
    int* launches;
};

int grid_for(long long work, int per_cta, int cap) {
    long long g = (work + per_cta - 1) / per_cta;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}

// Sorts every listed group (key, W) in place in compact slot space.
void sort_groups(Storage* S, const int* host_counts, uint32_t* key, int* W, const Launch& L) {
    FwdBuffers& f = S->f;
    int* cnt = S->counters;
    int nsm = host_counts[CNT_SMALL], nmd = host_counts[CNT_MED], nlg = host_counts[CNT_LARGE];
    if (nsm > 0) {
        k_sort_small<<<grid_for(nsm, kThreads, L.sms * 16), kThreads, 0, L.st>>>(f.list[0], cnt + CNT_SMALL, key, W);
        QZ_DBG(L.st, "k_sort_small");
        ++*L.launches;
    }
    if (nmd > 0) {
        k_sort_medium<<<grid_for(nmd, 1, L.sms * 4), kThreads, 0, L.st>>>(f.list[1], cnt + CNT_MED, key, W);
        QZ_DBG(L.st, "k_sort_medium");
        ++*L.launches;
    }
    if (nlg > 0) {
        k_large_prep<<<grid_for(nlg, kThreads, L.sms * 4), kThreads, 0, L.st>>>(f.list[2], cnt + CNT_LARGE, f.ltc,
                                                                                 f.llen);
        QZ_DBG(L.st, "k_large_prep");
        ++*L.launches;
        scan_exclusive(f.ltc, f.ltbase, 0, cnt + CNT_LARGE, S->partial, (uint32_t*)(cnt + CNT_LTILES), L.st,
                       L.launches);
        scan_exclusive(f.llen, f.lwbase, 0, cnt + CNT_LARGE, S->partial, nullptr, L.st, L.launches);
        LargeArgs la{f.list[2], cnt + CNT_LARGE, f.ltbase, f.lwbase, cnt + CNT_LTILES, cnt + CNT_LHIST};
        // upper bound of tiles: every large group is > kMedMax >= kRT long
        int grid = L.sms * 4;
        const uint32_t* sk[4] = {key, f.wsk[0], f.wsk[1], f.wsk[0]};
        const int* sv[4] = {W, f.wsv[0], f.wsv[1], f.wsv[0]};
        uint32_t* dk[4] = {f.wsk[0], f.wsk[1], f.wsk[0], key};
        int* dv[4] = {f.wsv[0], f.wsv[1], f.wsv[0], W};
        for (int pass = 0; pass < 4; ++pass) {
            int shift = 8 * pass;
            k_large_up<<<grid, kThreads, 0, L.st>>>(la, sk[pass], pass == 0, shift, S->hist);
            QZ_DBG(L.st, "k_large_up");
            ++*L.launches;
            // histogram entries = 256 * tiles (count on device)
            scan_exclusive(S->hist, S->hist, 0, cnt + CNT_LHIST, S->partial, nullptr, L.st, L.launches);
            k_large_down<<<grid, kThreads, 0, L.st>>>(la, S->hist, sk[pass], sv[pass], pass == 0, dk[pass],
                                                      dv[pass], pass == 3, shift);
            QZ_DBG(L.st, "k_large_down");
            ++*L.launches;
        }
    }
}

}  // namespace

int forward_run(Storage* S, int nb, const int* n, const uint8_t* d_T, uint8_t* d_U, int* idx,
                const int* aux_rate, int* aux_out, cudaStream_t st) {
    if (nb < 0 || nb > S->cap_blocks) return QZGPU_BAD_PARAMETER;
    long long N = 0;
    for (int b = 0; b < nb; ++b) {
        if (n[b] < 0) return QZGPU_BAD_PARAMETER;
        N += n[b];
    }
    if (N > S->cap_bytes) return QZGPU_BAD_PARAMETER;
    S->stats = qzgpu_stats{};
    S->rounds_active.clear();
    for (int b = 0; b < nb; ++b) idx[b] = n[b] <= 1 ? n[b] : -1;
    if (N == 0) return QZGPU_NO_ERROR;

    int launches = 0;
    Launch L{st, S->sms, &launches};
    FwdBuffers& f = S->f;

    // ---- host tables (pinned) -> device in one copy
    std::vector<int> off(nb + 1, 0);
    for (int b = 0; b < nb; ++b) off[b + 1] = off[b] + n[b];
    std::vector<int2> tiles;
    tiles.reserve((size_t)(N / kInitTile) + nb + 1);
    for (int b = 0; b < nb; ++b)
        for (int s = off[b]; s < off[b + 1]; s += kInitTile) tiles.push_back(make_int2(b, s));
    std::vector<int2> l0, l1, l2;
    for (int b = 0; b < nb; ++b) {
        if (n[b] < 2) continue;
        int2 dsc = make_int2(off[b], n[b]);
        if (n[b] <= kSmallMax) l0.push_back(dsc);
        else if (n[b] <= kMedMax) l1.push_back(dsc);
        else l2.push_back(dsc);
    }
    int aux_total = 0;
    std::vector<int> aoff(nb, 0);
    if (aux_rate) {
        for (int b = 0; b < nb; ++b) {
            aoff[b] = aux_total;
            if (aux_rate[b] > 0 && n[b] > 0) aux_total += (n[b] - 1) / aux_rate[b];
        }
    }
    // pinned layout: off | tiles | lists | counters | aux_rate | aux_off
    size_t need = sizeof(int) * (nb + 1) + sizeof(int2) * (tiles.size() + l0.size() + l1.size() + l2.size()) +
                  sizeof(int) * CNT_SLOTS + sizeof(int) * 2 * nb + 64;
    if (need > S->pin_tab_bytes || aux_total > 64 * S->cap_blocks) return QZGPU_BAD_PARAMETER;
    char* p = S->pin_tab;
    auto put = [&](const void* src, size_t bytes) {
        char* at = p;
        if (bytes) memcpy(p, src, bytes);
        p += (bytes + 15) / 16 * 16;
        return at;
    };
    char* h_off = put(off.data(), sizeof(int) * off.size());
    char* h_tiles = put(tiles.data(), sizeof(int2) * tiles.size());
    char* h_l0 = put(l0.data(), sizeof(int2) * l0.size());
    char* h_l1 = put(l1.data(), sizeof(int2) * l1.size());
    char* h_l2 = put(l2.data(), sizeof(int2) * l2.size());
    int cnt0[CNT_SLOTS] = {0};
    cnt0[CNT_ACTIVE] = (int)N;
    cnt0[CNT_SMALL] = (int)l0.size();
    cnt0[CNT_MED] = (int)l1.size();
    cnt0[CNT_LARGE] = (int)l2.size();
    char* h_cnt = put(cnt0, sizeof(cnt0));
    char* h_ar = aux_rate ? put(aux_rate, sizeof(int) * nb) : nullptr;
    char* h_ao = aux_rate ? put(aoff.data(), sizeof(int) * nb) : nullptr;
    cudaError_t e;
    auto h2d = [&](void* dst, const char* src, size_t bytes) {
        if (bytes && e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    };
    e = cudaSuccess;
    h2d(S->blk_off, h_off, sizeof(int) * off.size());
    h2d(S->tiles, h_tiles, sizeof(int2) * tiles.size());
    h2d(f.list[0], h_l0, sizeof(int2) * l0.size());
    h2d(f.list[1], h_l1, sizeof(int2) * l1.size());
    h2d(f.list[2], h_l2, sizeof(int2) * l2.size());
    h2d(S->counters, h_cnt, sizeof(cnt0));
    if (aux_rate) {
        h2d(S->blk_aux_rate, h_ar, sizeof(int) * nb);
        h2d(S->blk_aux_off, h_ao, sizeof(int) * nb);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(S->blk_hist, 0, sizeof(uint32_t) * 256 * nb, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(S->status, 0, sizeof(DevStatus), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(S->blk_idx, 0xff, sizeof(int) * nb, st);
    if (e != cudaSuccess) return map_cuda_error(e);

    // ---- alphabet, initial keys
    int ntiles = (int)tiles.size();
    k_block_hist<<<ntiles, kThreads, 0, st>>>(d_T, S->tiles, S->blk_off, S->blk_hist);
    QZ_DBG(st, "k_block_hist");
    k_block_alpha<<<nb, kThreads, 0, st>>>(S->blk_hist, S->blk_code, S->blk_K, S->blk_sigma);
    QZ_DBG(st, "k_block_alpha");
    k_init_keys<<<ntiles, kThreads, 0, st>>>(d_T, S->tiles, S->blk_off, S->blk_code, S->blk_K, S->blk_sigma, f.key,
                                             f.W[0], f.G[0]);
    QZ_DBG(st, "k_init_keys");
    launches += 3;

    const bool dump = dump_on() && N <= (1 << 20);
    if (dump) {
        dump_array("init_key", f.key, 4 * N, st);
        dump_array("init_W", f.W[0], 4 * N, st);
        dump_array("init_G", f.G[0], 4 * N, st);
        dump_array("blk_K", S->blk_K, 4 * nb, st);
        dump_array("blk_sigma", S->blk_sigma, 4 * nb, st);
    }
    // ---- initial sort (groups = blocks) and split
    int hc[CNT_SLOTS];
    memcpy(hc, cnt0, sizeof(hc));
    sort_groups(S, hc, f.key, f.W[0], L);
    if (dump) {
        dump_array("sorted_key", f.key, 4 * N, st);
        dump_array("sorted_W", f.W[0], 4 * N, st);
    }
    int cur = 0;
    int act = CNT_ACTIVE;  // counter slot holding the current active count
    auto split = [&](const int* P) {
        SplitArgs a;
        a.A = S->counters + act;
        a.A_next = S->counters + (act ^ (CNT_ACTIVE ^ CNT_ACTIVE_ALT));
        a.key = f.key;
        a.G = f.G[cur];
        a.P = P;
        a.W = f.W[cur];
        a.R = f.R;
        a.SA = f.SA;
        a.Pn = f.P[cur ^ 1];
        a.Wn = f.W[cur ^ 1];
        a.Gn = f.G[cur ^ 1];
        a.list0 = f.list[0];
        a.list1 = f.list[1];
        a.list2 = f.list[2];
        a.counters = S->counters;
        a.part_surv = S->split_part;
        a.part_head = S->split_part + kSplitGrid;
        k_split_count<<<kSplitGrid, kThreads, 0, st>>>(a);
        QZ_DBG(st, "k_split_count");
        k_split_top<<<1, kThreads, 0, st>>>(a);
        QZ_DBG(st, "k_split_top");
        k_split_apply<<<kSplitGrid, kThreads, 0, st>>>(a);
        QZ_DBG(st, "k_split_apply");
        launches += 3;
        cur ^= 1;
        act ^= CNT_ACTIVE ^ CNT_ACTIVE_ALT;
    };
    split(nullptr);
    auto dump_split = [&]() {
        if (!dump) return;
        dump_array("split_counters", S->counters, 4 * CNT_SLOTS, st);
        dump_array("split_R", f.R, 4 * N, st);
        dump_array("split_SA", f.SA, 4 * N, st);
        dump_array("split_P", f.P[cur], 4 * N, st);
        dump_array("split_W", f.W[cur], 4 * N, st);
        dump_array("split_G", f.G[cur], 4 * N, st);
        dump_array("split_list0", f.list[0], 8 * N / 2, st);
        dump_array("split_list1", f.list[1], 8 * (N / 17 + 1), st);
        dump_array("split_part", S->split_part, 4 * 2 * kSplitGrid, st);
    };
    dump_split();
    S->rounds_active.push_back((int)N);

    int* hcnt = S->pin_rd;
    int round = 0;
    for (;;) {
        e = cudaMemcpyAsync(hcnt, S->counters, sizeof(int) * CNT_SLOTS, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return map_cuda_error(e);
        int A = hcnt[act];
        if (A == 0) break;
        if (debug_on())
            debug_log("round %d: active %d small %d medium %d large %d", round, A, hcnt[CNT_SMALL], hcnt[CNT_MED],
                      hcnt[CNT_LARGE]);
        if (round >= kMaxRounds) {
            if (debug_on()) debug_log("no convergence after %d rounds", round);
            return QZGPU_GPU_ERROR;
        }
        S->rounds_active.push_back(A);
        k_gather<<<grid_for(A, kThreads, S->sms * 16), kThreads, 0, st>>>(S->counters + act, f.W[cur], f.R,
                                                                          S->blk_off, nb, S->blk_K, round, f.key);
        QZ_DBG(st, "k_gather");
        ++launches;
        if (dump) dump_array("gather_key", f.key, 4 * (size_t)A, st);
        sort_groups(S, hcnt, f.key, f.W[cur], L);
        if (dump) {
            dump_array("rsorted_key", f.key, 4 * (size_t)A, st);
            dump_array("rsorted_W", f.W[cur], 4 * (size_t)A, st);
        }
        split(f.P[cur]);
        dump_split();
        ++round;
    }

    // ---- U and primary indexes
    k_extract<<<grid_for(N, kThreads, S->sms * 16), kThreads, 0, st>>>(
        (int)N, f.SA, f.R, d_T, S->blk_off, nb, d_U, S->blk_idx, aux_rate ? S->blk_aux_rate : nullptr,
        S->blk_aux_off, S->aux, S->status);
    QZ_DBG(st, "k_extract");
    ++launches;
    DevStatus& hst = *reinterpret_cast<DevStatus*>(S->pin_rd + S->cap_blocks + 64);
    e = cudaMemcpyAsync(hcnt, S->blk_idx, sizeof(int) * nb, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hst, S->status, sizeof(hst), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && aux_out && aux_total)
        e = cudaMemcpyAsync(aux_out, S->aux, sizeof(int) * aux_total, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return map_cuda_error(e);
    if (hst.error) {
        if (debug_on()) debug_log("device status %d at %d detail %lld", hst.error, hst.where, hst.detail);
        return hst.error;
    }
    for (int b = 0; b < nb; ++b) {
        if (n[b] >= 2) {
            if (hcnt[b] < 1 || hcnt[b] > n[b]) {
                if (debug_on()) debug_log("block %d: primary index %d out of range (n %d)", b, hcnt[b], n[b]);
                return QZGPU_GPU_ERROR;
            }
            idx[b] = hcnt[b];
        }
    }
    long long active_sum = 0;
    for (int a : S->rounds_active) active_sum += a;
    S->stats.rounds = round;
    S->stats.kernel_launches = launches;
    S->stats.active_total = active_sum;
    S->stats.alg_bytes = 15 * N + 28 * active_sum;
    return QZGPU_NO_ERROR;
}

}  // namespace qz
