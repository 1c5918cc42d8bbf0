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
// Groups are kept in a compact work list in SA order (slot arrays W =
// suffix, G = group rank); a slot's SA position is G plus its offset in the
// group.  Per round each group is sorted by the kernel of its size class:
// <= 16 slots by rank counting in warp windows during the key gather (found
// from G, no list), 17..64 by rank counting in one warp, 65..512 by a warp
// radix sort, <= 4096 in one CTA's shared memory, larger ones by a segmented
// LSD radix sort over the whole GPU (radix.cu).  Round 0 gathers text keys
// (R holds them until round 0's split), so the initial split writes no ranks.
#include "engine.h"
#include "radix.cuh"
#include "scan.cuh"

namespace qz {


// ------------------------------------------------------------------ per-block alphabet

__global__ void __launch_bounds__(kThreads) k_block_hist(const uint8_t* __restrict__ T,
                                                         const int2* __restrict__ tiles, int ntiles,
                                                         const int* __restrict__ off,
                                                         uint32_t* __restrict__ bhist) {
    // each CTA counts a contiguous run of tiles into per-warp shared
    // histograms, all of a tile's bytes loaded before counting, and flushes
    // when the block changes
    __shared__ uint32_t h[kWarps][256];
    int lo, hi;
    chunk_range(ntiles, gridDim.x, blockIdx.x, 1, &lo, &hi);
    if (lo >= hi) return;
#pragma unroll
    for (int q = 0; q < kWarps; ++q) h[q][threadIdx.x] = 0;
    __syncthreads();
    constexpr int kPer = kInitTile / kThreads;
    int cur = tiles[lo].x;
    for (int t = lo; t < hi; ++t) {
        const int2 tl = tiles[t];
        if (tl.x != cur) {  // uniform across the CTA
            __syncthreads();
            uint32_t v = 0;
#pragma unroll
            for (int q = 0; q < kWarps; ++q) {
                v += h[q][threadIdx.x];
                h[q][threadIdx.x] = 0;
            }
            if (v) atomicAdd(&bhist[(size_t)cur * 256 + threadIdx.x], v);
            cur = tl.x;
            __syncthreads();
        }
        const int end = min(off[tl.x + 1], tl.y + kInitTile);
        unsigned c[kPer];
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            const int x = tl.y + k * kThreads + threadIdx.x;
            c[k] = x < end ? (unsigned)__ldcs(T + x) : 256u;
        }
#pragma unroll
        for (int k = 0; k < kPer; ++k)
            if (c[k] < 256u) atomicAdd(&h[warp_id()][c[k]], 1u);
    }
    __syncthreads();
    uint32_t v = 0;
#pragma unroll
    for (int q = 0; q < kWarps; ++q) v += h[q][threadIdx.x];
    if (v) atomicAdd(&bhist[(size_t)cur * 256 + threadIdx.x], v);
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
                                                        int* __restrict__ G, uint32_t* __restrict__ R) {
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
        R[x] = (uint32_t)k;
        W[x] = x;
        G[x] = bstart;
    }
}

// ------------------------------------------------------------------ rank gather

// Secondary key of suffix x in doubling round `round` (h = K_b << round):
// R[x+h] + h + 1 when x+h is inside the block, else the remaining length
// (n_b - i), which is <= h and orders the shorter suffix first.
//
// Round 0 reads text keys instead of ranks: R still holds the K_b-symbol key
// of every position (written by the initial key pass, not yet overwritten by
// any split), so the secondary key is R[x+h] itself, and a suffix that ends
// inside the window gets 0.  The key of x+h orders like its rank did; an
// ending suffix ties only with suffixes of its group whose next K_b symbols
// are all the smallest symbol (or padding).  Those ties form the first
// subgroup of the group in true suffix order and are broken by the end keys
// of the next round.  A block whose window covers it whole (h >= n_b: one
// symbol, or a block shorter than K_b) keeps the remaining-length key.
struct GatherArgs {
    const int* R;
    const int* off;
    int nb;
    const int* Kb;
    int round;
};

struct BlockSpan {
    int bs, n;
    long long h;
};

__device__ __forceinline__ BlockSpan block_span(const GatherArgs& g, int x) {
    int b = block_of(g.off, g.nb, x);
    BlockSpan s;
    s.bs = __ldg(g.off + b);
    s.n = __ldg(g.off + b + 1) - s.bs;
    s.h = g.round >= 31 ? (long long)s.n : ((long long)__ldg(g.Kb + b) << g.round);
    if (s.h > s.n) s.h = s.n;
    return s;
}

__device__ __forceinline__ uint32_t rank_key(const GatherArgs& g, const BlockSpan& s, int x) {
    int i = x - s.bs;
    if (g.round == 0) {
        if ((long long)i + s.h < s.n) return (uint32_t)ld_keep(g.R + x + (int)s.h, l2_keep_policy());
        return s.h >= s.n ? (uint32_t)(s.n - i) : 0u;
    }
    if ((long long)i + s.h < s.n) return (uint32_t)ld_keep(g.R + x + (int)s.h, l2_keep_policy()) + (uint32_t)s.h + 1u;
    return (uint32_t)(s.n - i);
}

// ------------------------------------------------------------------ group sorts

__device__ __forceinline__ unsigned long long pack_kv(uint32_t k, int v) {
    return ((unsigned long long)k << 32) | (uint32_t)v;
}

template <int M>
__device__ __forceinline__ void bitonic_regs(unsigned long long (&v)[M]) {
#pragma unroll
    for (int k = 2; k <= M; k <<= 1) {
#pragma unroll
        for (int jj = k >> 1; jj > 0; jj >>= 1) {
#pragma unroll
            for (int a = 0; a < M; ++a) {
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
}

template <int M>
__device__ __forceinline__ void sort_group_regs(int s, int len, uint32_t* key, int* W) {
    unsigned long long v[M];
#pragma unroll
    for (int j = 0; j < M; ++j) v[j] = j < len ? pack_kv(key[s + j], W[s + j]) : ~0ull;
    bitonic_regs<M>(v);
#pragma unroll
    for (int j = 0; j < M; ++j) {
        if (j < len) {
            key[s + j] = (uint32_t)(v[j] >> 32);
            W[s + j] = (int)(uint32_t)v[j];
        }
    }
}

// Groups of 2..16 slots.  Each warp takes a window of 32 consecutive slots;
// group bounds come from ballots over the group ranks G, and every lane of a
// group that lies inside the window computes its own rank in the group by
// counting smaller keys (ties broken by slot), then writes its key and suffix
// to that position.  A group that straddles the window end is sorted by the
// thread holding its first slot, in registers.
__global__ void __launch_bounds__(kThreads) k_sort_small(const int* __restrict__ d_A, const int* __restrict__ G,
                                                         uint32_t* __restrict__ key, int* __restrict__ W) {
    const int A = *d_A;
    const int ln = (int)lane_id();
    const int nwin = (A + 31) / 32;
    const int nwarps = gridDim.x * kWarps;
    for (int win = blockIdx.x * kWarps + (int)warp_id(); win < nwin; win += nwarps) {
        const int base = win * 32;
        const int k = base + ln;
        const bool valid = k < A;
        int g = valid ? G[k] : -1;
        int gp = __shfl_up_sync(0xffffffffu, g, 1);
        if (ln == 0) gp = (base > 0) ? G[base - 1] : -2;
        int gn = __shfl_down_sync(0xffffffffu, g, 1);
        if (ln == 31) gn = (k + 1 < A) ? G[k + 1] : -2;
        const bool head = valid && gp != g;
        const bool tail = valid && (k + 1 >= A || gn != g);
        const unsigned H = __ballot_sync(0xffffffffu, head);
        const unsigned T = __ballot_sync(0xffffffffu, tail);
        // group start: highest head at or below this lane; end: lowest tail at or above
        const unsigned hb = H & (0xffffffffu >> (31 - ln));
        const unsigned tb = T & (0xffffffffu << ln);
        const int s = hb ? 31 - __clz(hb) : -1;
        const int e = tb ? __ffs(tb) - 1 : 32;
        const bool inside = valid && s >= 0 && e < 32;
        const int L = inside ? e - s + 1 : 0;
        const bool mine = inside && L >= 2 && L <= kSmallMax;
        // only lanes of groups sorted here read their key and suffix
        uint32_t kv = mine ? key[k] : 0u;
        int wv = mine ? W[k] : 0;
        // every lane runs the same number of shuffles (the longest group in the window)
        int maxL = mine ? L : 0;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) maxL = max(maxL, __shfl_xor_sync(0xffffffffu, maxL, d));
        int rank = 0;
        for (int j = 0; j < maxL; ++j) {
            int src = (mine ? s : 0) + j;
            uint32_t kj = __shfl_sync(0xffffffffu, kv, src & 31);
            if (mine && j < L) rank += (kj < kv || (kj == kv && src < ln)) ? 1 : 0;
        }
        if (mine) {
            key[base + s + rank] = kv;
            W[base + s + rank] = wv;
        }
        // a group that starts in this window and ends after it
        if (head && !(T & (0xffffffffu << ln))) {
            int L2 = 32 - ln;
            while (L2 <= kSmallMax && k + L2 < A && G[k + L2] == g) ++L2;
            if (L2 >= 2 && L2 <= kSmallMax) {
                if (L2 <= 4) sort_group_regs<4>(k, L2, key, W);
                else if (L2 <= 8) sort_group_regs<8>(k, L2, key, W);
                else sort_group_regs<16>(k, L2, key, W);
            }
        }
    }
}

// Doubling rounds: secondary keys of all active slots, with groups of 2..16
// slots sorted on the spot.  Each warp takes a run of kGatherRun consecutive
// 32-slot windows.  Each lane gathers the key of its slot; group bounds come
// from ballots over G; a lane of an in-window small group takes its rank in
// the group by counting smaller keys (ties by slot) and writes key and suffix
// there.  Every other slot gets its key written in place (sorted later by its
// class).  A small group that crosses the boundary between two windows of the
// run is then re-ranked from the registers of both windows (it lies in the
// 32-slot window centred on the boundary); boundaries between runs are
// flagged for k_sort_straddle.
constexpr int kGatherRun = 8;

__device__ __forceinline__ void rank_centred(uint32_t ck, int cx, int cs, int L, int cbase, uint32_t* __restrict__ key,
                                             int* __restrict__ W) {
    const int ln = (int)lane_id();
    const bool m = ln >= cs && ln < cs + L;
    int r = 0;
    for (int j = 0; j < L; ++j) {
        uint32_t kj = __shfl_sync(0xffffffffu, ck, cs + j);
        if (m) r += (kj < ck || (kj == ck && cs + j < ln)) ? 1 : 0;
    }
    if (m) {
        key[cbase + cs + r] = ck;
        W[cbase + cs + r] = cx;
    }
}

__global__ void __launch_bounds__(kThreads) k_gather_small(const int* __restrict__ d_A, const int* __restrict__ G,
                                                           uint32_t* __restrict__ key, int* __restrict__ W,
                                                           GatherArgs ga, uint8_t* __restrict__ straddle) {
    const int A = *d_A;
    const int ln = (int)lane_id();
    const int nwin = (A + 31) / 32;
    const int nruns = (nwin + kGatherRun - 1) / kGatherRun;
    const int nwarps = gridDim.x * kWarps;
    for (int run = blockIdx.x * kWarps + (int)warp_id(); run < nruns; run += nwarps) {
        const int w_begin = run * kGatherRun, w_end = min(nwin, w_begin + kGatherRun);
        uint32_t pkv = 0;
        int px = 0, ps = 32;
        bool ptail = false;
        for (int win = w_begin; win < w_end; ++win) {
            const int base = win * 32;
            const int k = base + ln;
            const bool valid = k < A;
            int g = valid ? G[k] : -1;
            int x = valid ? W[k] : 0;
            int gp = __shfl_up_sync(0xffffffffu, g, 1);
            if (ln == 0) gp = (base > 0) ? G[base - 1] : -2;
            int gn = __shfl_down_sync(0xffffffffu, g, 1);
            if (ln == 31) gn = (k + 1 < A) ? G[k + 1] : -2;
            uint32_t kv = 0;
            if (valid) kv = rank_key(ga, block_span(ga, x), x);
            const unsigned H = __ballot_sync(0xffffffffu, valid && gp != g);
            const unsigned T = __ballot_sync(0xffffffffu, valid && (k + 1 >= A || gn != g));
            const unsigned hb = H & (0xffffffffu >> (31 - ln));
            const unsigned tb = T & (0xffffffffu << ln);
            const int s = hb ? 31 - __clz(hb) : -1;
            const int e = tb ? __ffs(tb) - 1 : 32;
            const bool inside = valid && s >= 0 && e < 32;
            const int L = inside ? e - s + 1 : 0;
            const bool mine = inside && L >= 2 && L <= kSmallMax;
            int maxL = mine ? L : 0;
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) maxL = max(maxL, __shfl_xor_sync(0xffffffffu, maxL, d));
            int rank = 0;
            for (int j = 0; j < maxL; ++j) {
                int src = (mine ? s : 0) + j;
                uint32_t kj = __shfl_sync(0xffffffffu, kv, src & 31);
                if (mine && j < L) rank += (kj < kv || (kj == kv && src < ln)) ? 1 : 0;
            }
            if (mine) {
                __stcs(key + base + s + rank, kv);
                __stcs(W + base + s + rank, x);
            } else if (valid) {
                __stcs(key + k, kv);
            }
            // the previous window's last group continues here: if it is small
            // it lies in the centred window (previous lanes 16..31, these 0..15)
            if (ptail) {
                const int e0 = T ? __ffs(T) - 1 : 32;
                const int Lc = (32 - ps) + e0 + 1;
                if (e0 < 16 && Lc <= kSmallMax) {
                    __syncwarp();
                    const uint32_t a = __shfl_sync(0xffffffffu, pkv, (ln + 16) & 31);
                    const uint32_t b = __shfl_sync(0xffffffffu, kv, (ln + 16) & 31);
                    const int ax = __shfl_sync(0xffffffffu, px, (ln + 16) & 31);
                    const int bx = __shfl_sync(0xffffffffu, x, (ln + 16) & 31);
                    rank_centred(ln < 16 ? a : b, ln < 16 ? ax : bx, ps - 16, Lc, base - 16, key, W);
                }
            }
            // this window's last group runs on and started in its upper half
            const bool tail = __shfl_sync(0xffffffffu, valid && gn == g && s >= 16, 31);
            ps = __shfl_sync(0xffffffffu, s, 31);
            ptail = tail;
            pkv = kv;
            px = x;
            if (win == w_end - 1) {
                if (ln == 0) straddle[run] = tail ? 1 : 0;
            }
        }
    }
}

// Groups of 2..16 slots that cross the boundary after the last window of a
// gather run: each lies inside the 32-slot window centred on that boundary,
// where it is ranked as above.  Only flagged boundaries are visited.
__global__ void __launch_bounds__(kThreads) k_sort_straddle(const int* __restrict__ d_A, const int* __restrict__ G,
                                                            uint32_t* __restrict__ key, int* __restrict__ W,
                                                            const uint8_t* __restrict__ straddle) {
    const int A = *d_A;
    const int ln = (int)lane_id();
    const int nwin = (A + 31) / 32;
    const int nruns = (nwin + kGatherRun - 1) / kGatherRun;
    const int nwarps = gridDim.x * kWarps;
    for (int run = blockIdx.x * kWarps + (int)warp_id(); run < nruns; run += nwarps) {
        if (!straddle[run]) continue;  // uniform across the warp
        const int win = min(nwin, (run + 1) * kGatherRun) - 1;
        const int base = win * 32 + 16;
        const int k = base + ln;
        const bool valid = k < A;
        int g = valid ? G[k] : -1;
        int gp = __shfl_up_sync(0xffffffffu, g, 1);
        if (ln == 0) gp = G[base - 1];
        int gn = __shfl_down_sync(0xffffffffu, g, 1);
        if (ln == 31) gn = (k + 1 < A) ? G[k + 1] : -2;
        const unsigned H = __ballot_sync(0xffffffffu, valid && gp != g);
        const unsigned T = __ballot_sync(0xffffffffu, valid && (k + 1 >= A || gn != g));
        // the group holding lane 16 crosses the boundary if it starts below lane 16
        const unsigned h16 = H & 0x1ffffu;
        const unsigned t16 = T & 0xffff0000u;
        const int s = h16 ? 31 - __clz(h16) : -1;
        const int e = t16 ? __ffs(t16) - 1 : 32;
        const int L = e - s + 1;
        if (s < 0 || s >= 16 || e >= 32 || L > kSmallMax) continue;  // uniform across the warp
        const bool mine = ln >= s && ln <= e;
        uint32_t kv = mine ? key[k] : 0u;
        int wv = mine ? W[k] : 0;
        rank_centred(kv, wv, s, L, base, key, W);
    }
}

// 65..512 slots: LSD radix sort by one warp.  Lane l holds slots it*32 + l
// in registers; each pass ranks them (256 digit counters in shared memory),
// scatters (key, suffix) pairs into the warp's one shared buffer and reads them
// back in the new order.  8-bit digits that are equal across the whole group
// are skipped.  The first pass run ranks with shared atomics (equal keys may
// leave in any order); the later ones are stable (warp matches).
constexpr size_t kMedWarpSmem = (size_t)kMedMax * 8 + 256 * 4;

__device__ __forceinline__ void warp_radix_sort(const uint32_t* skey, const int* sW, uint32_t* key, int* W, int s,
                                                int len, unsigned char* wsm) {
    unsigned long long* buf = reinterpret_cast<unsigned long long*>(wsm);
    uint32_t* cnt = reinterpret_cast<uint32_t*>(buf + kMedMax);
    const int ln = (int)lane_id();
    const unsigned lt = (1u << ln) - 1u;
    const int nit = (len + 31) >> 5;
    uint32_t kr[kMedMax / 32];
    int vr[kMedMax / 32];
    uint32_t kor = 0, kand = 0xffffffffu;
#pragma unroll
    for (int it = 0; it < kMedMax / 32; ++it) {
        const int i = it * 32 + ln;
        kr[it] = 0;
        vr[it] = 0;
        if (it < nit && i < len) {
            kr[it] = skey[s + i];
            vr[it] = sW[s + i];
            kor |= kr[it];
            kand &= kr[it];
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        kor |= __shfl_xor_sync(0xffffffffu, kor, d);
        kand &= __shfl_xor_sync(0xffffffffu, kand, d);
    }
    const uint32_t diff = kor ^ kand;
    bool first = true;  // the first pass run needs no stability
    for (int pass = 0; pass < 4; ++pass) {
        const int sh = 8 * pass;
        if (((diff >> sh) & 255u) == 0) continue;
        reinterpret_cast<uint4*>(cnt)[2 * ln] = make_uint4(0, 0, 0, 0);
        reinterpret_cast<uint4*>(cnt)[2 * ln + 1] = make_uint4(0, 0, 0, 0);
        __syncwarp();
        uint32_t rk[kMedMax / 32];
#pragma unroll
        for (int it = 0; it < kMedMax / 32; ++it) {
            if (it < nit) {
                const bool valid = it * 32 + ln < len;
                const unsigned dg = valid ? (kr[it] >> sh) & 255u : 256u;
                if (first) {
                    // equal keys may leave in any order: shared atomics rank
                    rk[it] = valid ? atomicAdd(&cnt[dg], 1u) : 0u;
                } else {
                    const unsigned peers = __match_any_sync(0xffffffffu, dg);
                    const unsigned before = __popc(peers & lt);
                    const uint32_t prev = valid ? cnt[dg] : 0u;
                    __syncwarp();
                    if (valid && before == 0) cnt[dg] = prev + __popc(peers);
                    __syncwarp();
                    rk[it] = prev + before;
                }
            }
        }
        __syncwarp();
        first = false;
        {
            // exclusive scan of the counters, eight consecutive digits per lane
            uint4 a = reinterpret_cast<uint4*>(cnt)[2 * ln], b = reinterpret_cast<uint4*>(cnt)[2 * ln + 1];
            uint32_t t0 = a.x, t1 = t0 + a.y, t2 = t1 + a.z, t3 = t2 + a.w;
            uint32_t t4 = t3 + b.x, t5 = t4 + b.y, t6 = t5 + b.z, t7 = t6 + b.w;
            uint32_t ex = warp_incl_sum(t7) - t7;
            reinterpret_cast<uint4*>(cnt)[2 * ln] = make_uint4(ex, ex + t0, ex + t1, ex + t2);
            reinterpret_cast<uint4*>(cnt)[2 * ln + 1] = make_uint4(ex + t3, ex + t4, ex + t5, ex + t6);
        }
        __syncwarp();
#pragma unroll
        for (int it = 0; it < kMedMax / 32; ++it) {
            if (it < nit && it * 32 + ln < len) {
                const uint32_t p = cnt[(kr[it] >> sh) & 255u] + rk[it];
                buf[p] = ((unsigned long long)kr[it] << 32) | (uint32_t)vr[it];
            }
        }
        __syncwarp();
#pragma unroll
        for (int it = 0; it < kMedMax / 32; ++it) {
            if (it < nit && it * 32 + ln < len) {
                const unsigned long long v = buf[it * 32 + ln];
                kr[it] = (uint32_t)(v >> 32);
                vr[it] = (int)(uint32_t)v;
            }
        }
        __syncwarp();
    }
#pragma unroll
    for (int it = 0; it < kMedMax / 32; ++it) {
        const int i = it * 32 + ln;
        if (it < nit && i < len) {
            key[s + i] = kr[it];
            W[s + i] = vr[it];
        }
    }
}

// Groups of up to 64 slots (the split lists 17..64 here), one warp per listed
// group: each slot ranks itself by counting smaller keys (ties by slot) over
// shuffled keys; one slot per lane up to 32 slots, two above.  The group is
// read from (skey, sW) and written to (key, W), which may be the same arrays.
__global__ void __launch_bounds__(kThreads) k_sort_rbc(const int2* __restrict__ list, const int* __restrict__ d_count,
                                                       const uint32_t* skey, const int* sW, uint32_t* key, int* W) {
    int cnt = *d_count;
    const int nwarps = gridDim.x * kWarps;
    const int ln = (int)lane_id();
    for (int i = blockIdx.x * kWarps + (int)warp_id(); i < cnt; i += nwarps) {
        int2 d = list[i];
        const int s = d.x, len = d.y;
        bool v0 = ln < len;
        uint32_t k0 = v0 ? skey[s + ln] : 0xffffffffu;
        int w0 = v0 ? sW[s + ln] : 0;
        int r0 = 0;
        if (len <= 32) {
            for (int j = 0; j < len; ++j) {
                uint32_t kj = __shfl_sync(0xffffffffu, k0, j);
                r0 += (kj < k0 || (kj == k0 && j < ln)) ? 1 : 0;
            }
            if (v0) {
                key[s + r0] = k0;
                W[s + r0] = w0;
            }
            continue;
        }
        bool v1 = ln + 32 < len;
        uint32_t k1 = v1 ? skey[s + ln + 32] : 0xffffffffu;
        int w1 = v1 ? sW[s + ln + 32] : 0;
        int r1 = 0;
        for (int j = 0; j < len; ++j) {
            uint32_t kj = __shfl_sync(0xffffffffu, j < 32 ? k0 : k1, j & 31);
            r0 += (kj < k0 || (kj == k0 && j < ln)) ? 1 : 0;
            r1 += (kj < k1 || (kj == k1 && j < ln + 32)) ? 1 : 0;
        }
        if (v0) {
            key[s + r0] = k0;
            W[s + r0] = w0;
        }
        if (v1) {
            key[s + r1] = k1;
            W[s + r1] = w1;
        }
    }
}

// Groups of 65..512 slots, one warp per listed group: warp_radix_sort.
__global__ void __launch_bounds__(kThreads, 3) k_sort_medium(const int2* __restrict__ list,
                                                          const int* __restrict__ d_count, const uint32_t* skey,
                                                          const int* sW, uint32_t* key, int* W) {
    extern __shared__ __align__(16) unsigned char msm[];
    int cnt = *d_count;
    const int nwarps = gridDim.x * kWarps;
    unsigned char* wsm = msm + warp_id() * kMedWarpSmem;
    for (int i = blockIdx.x * kWarps + (int)warp_id(); i < cnt; i += nwarps) {
        int2 d = list[i];
        warp_radix_sort(skey, sW, key, W, d.x, d.y, wsm);
    }
}

// ------------------------------------------------------------------ split into groups
//
// After a sort, slot k (compact, SA order) holds suffix W[k] of group G[k]
// (the group's rank = SA position of its first slot) with sort key key[k].
// A subgroup starts where G or key changes.  Each warp owns a tile of 256
// consecutive slots (lane l holds slots base + 32 i + l); per-tile partials
// (survivors, last subgroup head, last group head) are scanned across tiles
// so the apply pass needs no block-level synchronisation:
//   slot SA position  P = G + (k - first slot of the group)
//   new rank          = G + (first slot of the subgroup - first slot of the group)
// Singleton subgroups are final (SA[P] = suffix); the others are compacted,
// in order, into the next round's slot arrays.

constexpr int kWT = 256;  // slots per warp tile

// Rank writes of a split.  The initial split writes none (R keeps the text
// keys that round 0 gathers); round 0's split writes every slot's rank; later
// splits write the ranks that changed.
constexpr int kRankNone = 0, kRankChanged = 1, kRankAll = 2;
constexpr int kWI = kWT / 32;

struct SplitArgs {
    const int* A;      // active slots of this split
    int* A_next;       // receives the survivor count
    const uint32_t* key;
    const int* G;
    const int* W;
    int* R;
    int* SA;
    int* Wn;
    int* Gn;
    int2* list_rbc;
    int2* list_med;
    int2* list_tile;
    int2* list_large;
    int* counters;
    uint32_t* p_surv;  // per warp tile; exclusive prefix after the partial scan
    int* p_sub;
    int* p_grp;
    int write_rank;    // kRankNone / kRankChanged / kRankAll
    int medium_max;    // longest group listed for the one-warp sort
    int n;             // suffix-array entries (bound of the SA stores)
    DevStatus* st;
};

// Lane l of a warp tile holds the 8 consecutive slots base + 8l .. base + 8l + 7,
// so a slot's neighbours are in the lane's own registers except at its ends
// (one shuffle each way); flags are bit masks over the lane's 8 slots.
struct WarpTile {
    uint32_t k[kWI];
    int g[kWI];
    int w[kWI];
    unsigned valid, gh, sh, nsh;
};

template <typename T>
__device__ __forceinline__ void ld8(const T* __restrict__ p, int first, int A, T (&v)[kWI], T fill) {
    static_assert(sizeof(T) == 4 && kWI == 8, "two 16-byte loads per lane");
    if (first + kWI <= A) {
        // first is a multiple of 8 and the arrays start 256-byte aligned
        const uint4 a = __ldcs(reinterpret_cast<const uint4*>(p + first));
        const uint4 b = __ldcs(reinterpret_cast<const uint4*>(p + first + 4));
        const uint32_t u[kWI] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
        for (int i = 0; i < kWI; ++i) v[i] = (T)u[i];
    } else {
#pragma unroll
        for (int i = 0; i < kWI; ++i) v[i] = first + i < A ? __ldcs(p + first + i) : fill;
    }
}

template <bool WithSuffix>
__device__ __forceinline__ void wt_load(const SplitArgs& a, int A, int base, WarpTile& t) {
    const int ln = (int)lane_id();
    const int first = base + kWI * ln;
    ld8<uint32_t>(a.key, first, A, t.k, 0u);
    ld8<int>(a.G, first, A, t.g, -1);
    if (WithSuffix) ld8<int>(a.W, first, A, t.w, 0);
    uint32_t pk = __shfl_up_sync(0xffffffffu, t.k[kWI - 1], 1);
    int pg = __shfl_up_sync(0xffffffffu, t.g[kWI - 1], 1);
    uint32_t nk = __shfl_down_sync(0xffffffffu, t.k[0], 1);
    int ng = __shfl_down_sync(0xffffffffu, t.g[0], 1);
    if (ln == 0) {
        pk = base > 0 ? a.key[base - 1] : 0u;
        pg = base > 0 ? a.G[base - 1] : -1;
    }
    if (ln == 31) {
        nk = base + kWT < A ? a.key[base + kWT] : 0u;
        ng = base + kWT < A ? a.G[base + kWT] : -1;
    }
    t.valid = t.gh = t.sh = t.nsh = 0;
#pragma unroll
    for (int i = 0; i < kWI; ++i) {
        const int kk = first + i;
        const bool v = kk < A;
        const uint32_t prk = i > 0 ? t.k[i - 1] : pk;
        const int prg = i > 0 ? t.g[i - 1] : pg;
        const uint32_t nxk = i + 1 < kWI ? t.k[i + 1] : nk;
        const int nxg = i + 1 < kWI ? t.g[i + 1] : ng;
        const bool gh = v && (kk == 0 || prg != t.g[i]);
        const bool sh = v && (gh || prk != t.k[i]);
        const bool nsh = kk + 1 >= A || nxg != t.g[i] || nxk != t.k[i];
        t.valid |= (unsigned)v << i;
        t.gh |= (unsigned)gh << i;
        t.sh |= (unsigned)sh << i;
        t.nsh |= (unsigned)nsh << i;
    }
}

__global__ void __launch_bounds__(kThreads) k_split_count(SplitArgs a) {
    int A = *a.A;
    int ntiles = (A + kWT - 1) / kWT;
    int nwarps = gridDim.x * kWarps;
    for (int tile = blockIdx.x * kWarps + (int)warp_id(); tile < ntiles; tile += nwarps) {
        int base = tile * kWT;
        WarpTile t;
        wt_load<false>(a, A, base, t);
        const int first = base + kWI * (int)lane_id();
        uint32_t surv = __popc(t.valid & ~(t.sh & t.nsh));
        int sub = t.sh ? first + 31 - __clz(t.sh) : -1;
        int grp = t.gh ? first + 31 - __clz(t.gh) : -1;
        surv = warp_sum(surv);
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            sub = max(sub, __shfl_xor_sync(0xffffffffu, sub, d));
            grp = max(grp, __shfl_xor_sync(0xffffffffu, grp, d));
        }
        if (lane_id() == 0) {
            a.p_surv[tile] = surv;
            a.p_sub[tile] = sub;
            a.p_grp[tile] = grp;
        }
    }
}

// Exclusive scan of the per-tile partials (sum of survivors, max of the two
// head positions), reduce-then-scan over kScanGrid chunks.
__global__ void __launch_bounds__(kThreads) k_pscan_reduce(SplitArgs a, uint32_t* __restrict__ cs,
                                                           int* __restrict__ cm1, int* __restrict__ cm2) {
    __shared__ uint32_t shs[kWarps + 1];
    __shared__ int shm[kWarps + 1];
    int n = (*a.A + kWT - 1) / kWT;
    int lo, hi;
    chunk_range(n, gridDim.x, blockIdx.x, kThreads, &lo, &hi);
    uint32_t s = 0;
    int m1 = -1, m2 = -1;
    for (int i = lo + threadIdx.x; i < hi; i += kThreads) {
        s += a.p_surv[i];
        m1 = max(m1, a.p_sub[i]);
        m2 = max(m2, a.p_grp[i]);
    }
    uint32_t ts;
    block_excl_sum(s, shs, &ts);
    int t1, t2;
    block_incl_max(m1, shm, &t1);
    block_incl_max(m2, shm, &t2);
    if (threadIdx.x == 0) {
        cs[blockIdx.x] = ts;
        cm1[blockIdx.x] = t1;
        cm2[blockIdx.x] = t2;
    }
}

__device__ __forceinline__ int block_excl_max(int v, int* sh, int* total) {
    __shared__ int lastw[kWarps];
    int inc = block_incl_max(v, sh, total);
    int ex = __shfl_up_sync(0xffffffffu, inc, 1);
    if (lane_id() == 31) lastw[warp_id()] = inc;
    __syncthreads();
    if (lane_id() == 0) ex = warp_id() == 0 ? INT32_MIN : lastw[warp_id() - 1];
    __syncthreads();
    return ex;
}

__global__ void __launch_bounds__(kThreads) k_pscan_top(SplitArgs a, uint32_t* __restrict__ cs,
                                                        int* __restrict__ cm1, int* __restrict__ cm2, int n) {
    __shared__ uint32_t shs[kWarps + 1];
    __shared__ int shm[kWarps + 1];
    uint32_t carry = 0;
    int c1 = -1, c2 = -1;
    for (int base = 0; base < n; base += kThreads) {
        int i = base + threadIdx.x;
        uint32_t v = i < n ? cs[i] : 0u;
        int m1 = i < n ? cm1[i] : -1, m2 = i < n ? cm2[i] : -1;
        uint32_t tot;
        uint32_t ex = block_excl_sum(v, shs, &tot);
        int t1, t2;
        int e1 = block_excl_max(m1, shm, &t1);
        int e2 = block_excl_max(m2, shm, &t2);
        if (i < n) {
            cs[i] = carry + ex;
            cm1[i] = max(c1, e1);
            cm2[i] = max(c2, e2);
        }
        carry += tot;
        c1 = max(c1, t1);
        c2 = max(c2, t2);
    }
    if (threadIdx.x == 0) {
        *a.A_next = (int)carry;
    }
}

// Short rounds: one CTA scans all per-tile partials in place (what
// k_pscan_reduce, k_pscan_top and k_pscan_apply do together).
constexpr int kPscanSingleMax = 4096;  // warp tiles

__global__ void __launch_bounds__(kThreads) k_pscan_single(SplitArgs a) {
    __shared__ uint32_t shs[kWarps + 1];
    __shared__ int shm[kWarps + 1];
    const int n = (*a.A + kWT - 1) / kWT;
    uint32_t carry = 0;
    int c1 = -1, c2 = -1;
    for (int base = 0; base < n; base += kThreads) {
        const int i = base + threadIdx.x;
        const bool ok = i < n;
        const uint32_t v = ok ? a.p_surv[i] : 0u;
        const int m1 = ok ? a.p_sub[i] : -1, m2 = ok ? a.p_grp[i] : -1;
        uint32_t tot;
        const uint32_t ex = block_excl_sum(v, shs, &tot);
        int t1, t2;
        const int e1 = block_excl_max(m1, shm, &t1);
        const int e2 = block_excl_max(m2, shm, &t2);
        if (ok) {
            a.p_surv[i] = carry + ex;
            a.p_sub[i] = max(c1, e1);
            a.p_grp[i] = max(c2, e2);
        }
        carry += tot;
        c1 = max(c1, t1);
        c2 = max(c2, t2);
    }
    if (threadIdx.x == 0) {
        *a.A_next = (int)carry;
    }
}

__global__ void __launch_bounds__(kThreads) k_pscan_apply(SplitArgs a, const uint32_t* __restrict__ cs,
                                                          const int* __restrict__ cm1,
                                                          const int* __restrict__ cm2) {
    __shared__ uint32_t shs[kWarps + 1];
    __shared__ int shm[kWarps + 1];
    int n = (*a.A + kWT - 1) / kWT;
    int lo, hi;
    chunk_range(n, gridDim.x, blockIdx.x, kThreads, &lo, &hi);
    uint32_t carry = cs[blockIdx.x];
    int c1 = cm1[blockIdx.x], c2 = cm2[blockIdx.x];
    for (int base = lo; base < hi; base += kThreads) {
        int i = base + threadIdx.x;
        bool ok = i < hi;
        uint32_t v = ok ? a.p_surv[i] : 0u;
        int m1 = ok ? a.p_sub[i] : -1, m2 = ok ? a.p_grp[i] : -1;
        uint32_t tot;
        uint32_t ex = block_excl_sum(v, shs, &tot);
        int t1, t2;
        int e1 = block_excl_max(m1, shm, &t1);
        int e2 = block_excl_max(m2, shm, &t2);
        if (ok) {
            a.p_surv[i] = carry + ex;
            a.p_sub[i] = max(c1, e1);
            a.p_grp[i] = max(c2, e2);
        }
        carry += tot;
        c1 = max(c1, t1);
        c2 = max(c2, t2);
    }
}

// A loaded warp tile's per-lane counts: survivors and finished suffixes among
// the lane's slots with their inclusive scans over the lanes, the last
// subgroup and group heads of the lanes before it, and the tile's totals.
struct TileScan {
    unsigned alive;
    int lsurv, isurv, lsing, ising;
    int xsub, xgrp;  // exclusive over the lanes (-1: none)
    int tsurv, tsub, tgrp;
};

__device__ __forceinline__ TileScan tile_scan(const WarpTile& t, int first) {
    const int ln = (int)lane_id();
    TileScan s;
    s.alive = t.valid & ~(t.sh & t.nsh);
    s.lsurv = __popc(s.alive);
    const int lsub = t.sh ? first + 31 - __clz(t.sh) : -1;
    const int lgrp = t.gh ? first + 31 - __clz(t.gh) : -1;
    s.isurv = warp_incl_sum(s.lsurv);
    s.lsing = __popc(t.valid) - s.lsurv;
    s.ising = warp_incl_sum(s.lsing);
    const int isub = warp_incl_max(lsub), igrp = warp_incl_max(lgrp);
    s.xsub = __shfl_up_sync(0xffffffffu, isub, 1);
    s.xgrp = __shfl_up_sync(0xffffffffu, igrp, 1);
    if (ln == 0) s.xsub = s.xgrp = -1;
    s.tsurv = __shfl_sync(0xffffffffu, s.isurv, 31);
    s.tsub = __shfl_sync(0xffffffffu, isub, 31);
    s.tgrp = __shfl_sync(0xffffffffu, igrp, 31);
    return s;
}

// The stores of one warp tile, given the survivors of the tiles before it
// (dest) and the last subgroup and group heads before it (psub, pgrp).
__device__ __forceinline__ void split_tile_apply(const SplitArgs& a, const WarpTile& t, const TileScan& s,
                                                 int first, uint32_t dest, int psub, int pgrp, int2* st,
                                                 unsigned long long pol) {
    const int ln = (int)lane_id();
    int ks = max(psub, s.xsub), kg = max(pgrp, s.xgrp);
    int at = s.isurv - s.lsurv;   // this lane's first survivor, within the tile
    int atf = s.ising - s.lsing;  // this lane's first finished suffix, within the tile
#pragma unroll
    for (int i = 0; i < kWI; ++i) {
        if (!(t.valid >> i & 1u)) continue;
        const int kk = first + i;
        if (t.sh >> i & 1u) ks = kk;
        if (t.gh >> i & 1u) kg = kk;
        const int w = t.w[i], g = t.g[i];
        const int rank = g + (ks - kg);
        if (a.write_rank == kRankAll || (a.write_rank == kRankChanged && rank != g)) st_keep(a.R + w, rank, pol);
        if (!(s.alive >> i & 1u)) {
            st[kWT - 1 - atf] = make_int2(g + (kk - kg), w);
            ++atf;
            continue;
        }
        st[at] = make_int2(w, rank);
        const uint32_t d = dest + (uint32_t)at;
        ++at;
        // a surviving subgroup longer than kSmallMax ends here: list it by class
        const int L = kk - ks + 1;
        if ((t.nsh >> i & 1u) && L > kSmallMax) {
            const int cls = L <= 64 ? 3 : (L <= a.medium_max ? 0 : (L <= kOT ? 1 : 2));
            const int ci = cls == 0 ? CNT_MED : (cls == 1 ? CNT_TILE : (cls == 2 ? CNT_LARGE : CNT_PAIR));
            const int ce = cls == 0 ? CNT_MED_ELEMS
                                    : (cls == 1 ? CNT_TILE_ELEMS : (cls == 2 ? CNT_LARGE_ELEMS : CNT_PAIR_ELEMS));
            int2* list = cls == 0 ? a.list_med : (cls == 1 ? a.list_tile : (cls == 2 ? a.list_large : a.list_rbc));
            list[atomicAdd(&a.counters[ci], 1)] = make_int2((int)d - L + 1, L);
            atomicAdd(&a.counters[ce], L);
        }
    }
    __syncwarp();
    for (int j = ln; j < s.tsurv; j += 32) {
        const int2 v = st[j];
        __stcs(a.Wn + dest + j, v.x);
        __stcs(a.Gn + dest + j, v.y);
    }
    const int fin = __shfl_sync(0xffffffffu, s.ising, 31);
    for (int j = ln; j < fin; j += 32) {
        const int2 v = st[kWT - 1 - j];
        if ((unsigned)v.x < (unsigned)a.n) a.SA[v.x] = v.y;
    }
    __syncwarp();
}

__global__ void __launch_bounds__(kThreads, 5) k_split_apply(SplitArgs a) {
    // a warp tile's survivors (from the front) and finished suffixes (from the
    // back), staged so that both leave as coalesced rows
    __shared__ int2 stage[kWarps][kWT];
    if (failed(a.st)) return;  // suffixes may be duplicated or stale
    int A = *a.A;
    int ntiles = (A + kWT - 1) / kWT;
    int nwarps = gridDim.x * kWarps;
    int2* st = stage[warp_id()];
    const unsigned long long pol = l2_keep_policy();
    for (int tile = blockIdx.x * kWarps + (int)warp_id(); tile < ntiles; tile += nwarps) {
        const int base = tile * kWT;
        WarpTile t;
        wt_load<true>(a, A, base, t);
        const int first = base + kWI * (int)lane_id();
        const TileScan s = tile_scan(t, first);
        split_tile_apply(a, t, s, first, a.p_surv[tile], a.p_sub[tile], a.p_grp[tile], st, pol);
    }
}

// ------------------------------------------------------------------ one-pass split
//
// The count, scan and apply passes above in one pass over CTA tiles of
// kWarps warp tiles (2048 slots).  CTAs take tiles by ticket, in order.  Each
// warp loads and scans its warp tile; warp 0 combines the warps' totals
// (survivors, last subgroup head, last group head), publishes the tile's
// totals, looks back over the tiles before it for their exclusive values
// (decoupled look-back, one lane per earlier tile, 32 at a time) and
// publishes its inclusive values; then every warp applies its warp tile.
// Each total has its own status word per tile: the value in the low 32 bits,
// the state (1 aggregate, 2 inclusive) in bits 32-33 and the launch's epoch
// above, so nothing is cleared between splits.  Heads are stored plus one,
// so that zero means none.  A tile waits only on tiles of earlier tickets,
// which resident CTAs hold and publish before they wait; a wait that exceeds
// its limit records QZGPU_TIMEOUT, and the tile then stores nothing (its
// inclusive values are still published, so that the tiles after it finish).

constexpr int kCT = kWarps * kWT;  // slots per CTA tile of the one-pass split

struct SplitLookBack {
    unsigned long long* status;  // 4 words per CTA tile (3 used)
    unsigned* ticket;
    unsigned epoch;
    unsigned spin_limit;
    int silent_tile;  // failure-detection test: this tile publishes nothing (-1: none)
};

constexpr unsigned kSplitSpinLimit = 1u << 24;  // polls of 32 ns and more
constexpr unsigned long long kSplitAgg = 1ull << 32;
constexpr unsigned long long kSplitInc = 2ull << 32;

__device__ __forceinline__ bool split_ready(unsigned long long v, unsigned epoch) {
    return (unsigned)(v >> 34) == epoch && (v & (3ull << 32)) != 0;
}

// Exclusive totals of the tiles before `tile` (one warp): ex[0] survivors
// (sum), ex[1] and ex[2] last subgroup and group head plus one (max).  False
// if a wait ran out.
__device__ __forceinline__ bool split_look_back(const SplitLookBack& lb, int tile, uint32_t (&ex)[3],
                                                DevStatus* st) {
    const int ln = (int)lane_id();
    const unsigned long long none = ((unsigned long long)lb.epoch << 34) | kSplitInc;  // inclusive zero
    unsigned done = 0;  // bit c: total c found
    for (int p = tile - 1; done != 7u; p -= 32) {
        const int q = p - ln;  // this lane's tile
        const volatile unsigned long long* w = lb.status + 4ll * (q < 0 ? 0 : q);
        unsigned long long v[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) v[c] = (q >= 0 && !(done >> c & 1u)) ? w[c] : none;
        unsigned spins = 0;
        while (!(split_ready(v[0], lb.epoch) && split_ready(v[1], lb.epoch) && split_ready(v[2], lb.epoch)) &&
               spins < lb.spin_limit) {
            __nanosleep(32);
#pragma unroll
            for (int c = 0; c < 3; ++c)
                if (!split_ready(v[c], lb.epoch)) v[c] = w[c];
            ++spins;
        }
        if (__any_sync(0xffffffffu, spins >= lb.spin_limit)) {
            if (ln == 0) report(st, QZGPU_TIMEOUT, 21, tile);
            return false;
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (done >> c & 1u) continue;
            // lanes up to the nearest tile with an inclusive value contribute
            const unsigned inc = __ballot_sync(0xffffffffu, (v[c] & kSplitInc) != 0);
            const int lim = inc ? __ffs(inc) - 1 : 31;
            const unsigned x = ln <= lim ? (unsigned)v[c] : 0u;
            if (c == 0)
                ex[0] += __reduce_add_sync(0xffffffffu, x);
            else
                ex[c] = max(ex[c], __reduce_max_sync(0xffffffffu, x));
            if (inc) done |= 1u << c;
        }
    }
    return true;
}

__global__ void __launch_bounds__(kThreads, 5) k_split(SplitArgs a, SplitLookBack lb) {
    __shared__ int2 stage[kWarps][kWT];
    __shared__ uint32_t s_tot[3][kWarps];  // per warp tile: survivors, subgroup head + 1, group head + 1
    __shared__ uint32_t s_ex[3];           // the CTA tile's exclusive totals
    __shared__ int s_tile, s_ok;
    if (failed(a.st)) return;  // suffixes may be duplicated or stale
    const int A = *a.A;
    const int ntiles = (A + kCT - 1) / kCT;
    if (ntiles == 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) *a.A_next = 0;
        return;
    }
    const int ln = (int)lane_id(), wp = (int)warp_id();
    int2* st = stage[wp];
    const unsigned long long pol = l2_keep_policy();
    const unsigned long long ep = (unsigned long long)lb.epoch << 34;
    for (;;) {
        if (threadIdx.x == 0) s_tile = (int)atomicAdd(lb.ticket, 1u);
        __syncthreads();
        const int tile = s_tile;
        if (tile >= ntiles) return;
        const int base = tile * kCT + wp * kWT;
        const int first = base + kWI * ln;
        WarpTile t;
        if (base < A) {
            wt_load<true>(a, A, base, t);
        } else {
            t.valid = t.gh = t.sh = t.nsh = 0;
        }
        const TileScan s = tile_scan(t, first);
        if (ln == 0) {
            s_tot[0][wp] = (uint32_t)s.tsurv;
            s_tot[1][wp] = (uint32_t)(s.tsub + 1);
            s_tot[2][wp] = (uint32_t)(s.tgrp + 1);
        }
        __syncthreads();
        if (wp == 0) {
            // the CTA tile's totals and each warp tile's exclusive values within it
            const bool in = ln < kWarps;
            const uint32_t vs = in ? s_tot[0][ln] : 0u, vh = in ? s_tot[1][ln] : 0u, vg = in ? s_tot[2][ln] : 0u;
            const uint32_t is = warp_incl_sum(vs);
            const uint32_t ih = (uint32_t)warp_incl_max((int)vh), ig = (uint32_t)warp_incl_max((int)vg);
            const uint32_t agg0 = __shfl_sync(0xffffffffu, is, kWarps - 1);
            const uint32_t agg1 = __shfl_sync(0xffffffffu, ih, kWarps - 1);
            const uint32_t agg2 = __shfl_sync(0xffffffffu, ig, kWarps - 1);
            const uint32_t xh = __shfl_up_sync(0xffffffffu, ih, 1), xg = __shfl_up_sync(0xffffffffu, ig, 1);
            if (in) {
                s_tot[0][ln] = is - vs;
                s_tot[1][ln] = ln == 0 ? 0u : xh;
                s_tot[2][ln] = ln == 0 ? 0u : xg;
            }
            const uint32_t agg = ln == 0 ? agg0 : (ln == 1 ? agg1 : agg2);
            volatile unsigned long long* my = lb.status + 4ll * tile + ln;
            const bool pub = ln < 3 && tile != lb.silent_tile;
            uint32_t ex[3] = {0u, 0u, 0u};
            bool ok = true;
            if (tile > 0) {
                if (pub) *my = ep | kSplitAgg | agg;
                ok = split_look_back(lb, tile, ex, a.st);
            }
            const uint32_t mine = ln == 0 ? ex[0] : (ln == 1 ? ex[1] : ex[2]);
            if (pub) *my = ep | kSplitInc | (ln == 0 ? mine + agg : max(mine, agg));
            if (tile == ntiles - 1 && ln == 0) *a.A_next = (int)(ex[0] + agg0);
            if (ln == 0) {
                s_ex[0] = ex[0];
                s_ex[1] = ex[1];
                s_ex[2] = ex[2];
                s_ok = ok;
            }
        }
        __syncthreads();
        if (s_ok && base < A) {
            // survivors before a warp tile are at most its first slot
            const uint32_t dest = min(s_ex[0] + s_tot[0][wp], (uint32_t)base);
            const int psub = (int)max(s_ex[1], s_tot[1][wp]) - 1;
            const int pgrp = (int)max(s_ex[2], s_tot[2][wp]) - 1;
            split_tile_apply(a, t, s, first, dest, psub, pgrp, st, pol);
        }
        __syncthreads();  // s_tile, s_tot and s_ex are rewritten by the next tile
    }
}

// Ranks of the suffixes the initial split finished.  That split writes no
// ranks (R holds the text keys round 0 gathers), so once round 0 has gathered,
// every suffix-array entry it set (the others still hold -1) gives its suffix
// its final rank: the entry's position.
__global__ void __launch_bounds__(kThreads) k_rank_fixup(int N, const int* __restrict__ SA, int* __restrict__ R) {
    for (int j = blockIdx.x * kThreads + threadIdx.x; j < N; j += gridDim.x * kThreads) {
        int s = __ldcs(SA + j);
        if (s >= 0) st_keep(R + s, j, l2_keep_policy());
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

int grid_for(long long work, int per_cta, int cap) {
    long long g = (work + per_cta - 1) / per_cta;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}

}  // namespace

void sort_rbc_groups(Storage* S, const int2* list, const int* d_count, int host_count, long long elems,
                     const uint32_t* skey, const int* sval, uint32_t* key, int* val, cudaStream_t st) {
    if (host_count <= 0) return;
    QZ_LAUNCH(S, st, "k_sort_rbc", 16 * elems + 8ll * host_count,
              k_sort_rbc<<<grid_for(host_count, kWarps, S->sms * 16), kThreads, 0, st>>>(list, d_count, skey, sval,
                                                                                        key, val));
}

void sort_medium_groups(Storage* S, const int2* list, const int* d_count, int host_count, long long elems,
                        const uint32_t* skey, const int* sval, uint32_t* key, int* val, cudaStream_t st) {
    if (host_count <= 0) return;
    smem_limit_once<k_sort_medium>((int)(kWarps * kMedWarpSmem), S->device);
    QZ_LAUNCH(S, st, "k_sort_medium", 16 * elems + 8ll * host_count,
              k_sort_medium<<<grid_for(host_count, kWarps, S->sms * 16), kThreads, kWarps * kMedWarpSmem, st>>>(
                  list, d_count, skey, sval, key, val));
}

namespace {

// Sorts every group (key, W) in place in compact slot space.  hc: host copy
// of the counters (list lengths, slots per class); A: active slots.
void sort_groups(Storage* S, const int* hc, int A, const int* d_A, uint32_t* key, int* W, const int* G,
                 cudaStream_t st, bool small_done, int key_bits) {
    FwdBuffers& f = S->f;
    int* cnt = S->counters;
    const int sms = S->sms;
    long long small_el = (long long)A - hc[CNT_PAIR_ELEMS] - hc[CNT_MED_ELEMS] - hc[CNT_TILE_ELEMS] -
                         hc[CNT_LARGE_ELEMS];
    sort_rbc_groups(S, f.list_rbc, cnt + CNT_PAIR, hc[CNT_PAIR], hc[CNT_PAIR_ELEMS], key, W, key, W, st);
    // every slot: group rank read; small groups: key and suffix read and written
    if (small_el > 0 && !small_done)
        QZ_LAUNCH(S, st, "k_sort_small", 4ll * A + 16ll * small_el,
                  k_sort_small<<<grid_for(A, kThreads, sms * 16), kThreads, 0, st>>>(d_A, G, key, W));
    sort_medium_groups(S, f.list_med, cnt + CNT_MED, hc[CNT_MED], hc[CNT_MED_ELEMS], key, W, key, W, st);
    sort_tile_groups(S, f.list_tile, cnt + CNT_TILE, hc[CNT_TILE], hc[CNT_TILE_ELEMS], key, W, key, W, key_bits, st);
    sort_big_groups(S, f.list_large, cnt + CNT_LARGE, hc[CNT_LARGE], hc[CNT_LARGE_ELEMS], key, W, key_bits, st);
}

}  // namespace

namespace {

void add_round(Storage* S, int r, long long a) {
    if ((int)S->rounds_active.size() <= r) S->rounds_active.resize(r + 1, 0);
    S->rounds_active[r] += a;
}

// One sub-batch: blocks laid out back to back from d_T, using the storage
// arrays from position 0.  Accumulates round counts into S.
// Launches whose stores of survivors, suffix-array entries and ranks are known
// only once the next round's counts are read.
bool split_store_kernel(const char* name) {
    return strcmp(name, "k_split") == 0 || strcmp(name, "k_split_first") == 0 ||
           strncmp(name, "k_split_apply", 13) == 0;
}

int forward_core(Storage* S, int nb, const int* n, const uint8_t* d_T, uint8_t* d_U, int* idx,
                 const int* aux_rate, int* aux_out, cudaStream_t st, int* rounds_out) {
    long long N = 0;
    for (int b = 0; b < nb; ++b) N += n[b];
    for (int b = 0; b < nb; ++b) idx[b] = n[b] <= 1 ? n[b] : -1;
    if (N == 0) return QZGPU_NO_ERROR;
    FwdBuffers& f = S->f;

    // ---- host tables (pinned) -> device
    std::vector<int> off(nb + 1, 0);
    for (int b = 0; b < nb; ++b) off[b + 1] = off[b] + n[b];
    std::vector<int2> tiles;
    tiles.reserve((size_t)(N / kInitTile) + nb + 1);
    for (int b = 0; b < nb; ++b)
        for (int s = off[b]; s < off[b + 1]; s += kInitTile) tiles.push_back(make_int2(b, s));
    // initial groups = blocks; blocks of <= kSmallMax bytes need no list
    std::vector<int2> l0, l1, lt, l2;
    int cnt0[CNT_SLOTS] = {0};
    for (int b = 0; b < nb; ++b) {
        if (n[b] <= kSmallMax) continue;
        int2 dsc = make_int2(off[b], n[b]);
        if (n[b] <= 64) {
            l0.push_back(dsc);
            cnt0[CNT_PAIR_ELEMS] += n[b];
        } else if (n[b] <= S->tune.medium_max) {
            l1.push_back(dsc);
            cnt0[CNT_MED_ELEMS] += n[b];
        } else if (n[b] <= kOT) {
            lt.push_back(dsc);
            cnt0[CNT_TILE_ELEMS] += n[b];
        } else {
            l2.push_back(dsc);
            cnt0[CNT_LARGE_ELEMS] += n[b];
        }
    }
    int aux_total = 0;
    std::vector<int> aoff(nb, 0);
    if (aux_rate) {
        for (int b = 0; b < nb; ++b) {
            aoff[b] = aux_total;
            if (aux_rate[b] > 0 && n[b] > 0) aux_total += (n[b] - 1) / aux_rate[b];
        }
    }
    size_t need = sizeof(int) * (nb + 1) + sizeof(int2) * (tiles.size() + l0.size() + l1.size() + lt.size() + l2.size()) +
                  sizeof(int) * CNT_SLOTS + sizeof(int) * 2 * nb + 64 * 8;
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
    char* h_lt = put(lt.data(), sizeof(int2) * lt.size());
    char* h_l2 = put(l2.data(), sizeof(int2) * l2.size());
    cnt0[CNT_ACTIVE] = (int)N;
    cnt0[CNT_PAIR] = (int)l0.size();
    cnt0[CNT_MED] = (int)l1.size();
    cnt0[CNT_TILE] = (int)lt.size();
    cnt0[CNT_LARGE] = (int)l2.size();
    char* h_cnt = put(cnt0, sizeof(cnt0));
    char* h_ar = aux_rate ? put(aux_rate, sizeof(int) * nb) : nullptr;
    char* h_ao = aux_rate ? put(aoff.data(), sizeof(int) * nb) : nullptr;
    cudaError_t e = cudaSuccess;
    auto h2d = [&](void* dst, const char* src, size_t bytes) {
        if (bytes && e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    };
    h2d(S->blk_off, h_off, sizeof(int) * off.size());
    h2d(S->tiles, h_tiles, sizeof(int2) * tiles.size());
    h2d(f.list_rbc, h_l0, sizeof(int2) * l0.size());
    h2d(f.list_med, h_l1, sizeof(int2) * l1.size());
    h2d(f.list_tile, h_lt, sizeof(int2) * lt.size());
    h2d(f.list_large, h_l2, sizeof(int2) * l2.size());
    h2d(S->counters, h_cnt, sizeof(cnt0));
    if (aux_rate) {
        h2d(S->blk_aux_rate, h_ar, sizeof(int) * nb);
        h2d(S->blk_aux_off, h_ao, sizeof(int) * nb);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(S->blk_hist, 0, sizeof(uint32_t) * 256 * nb, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(S->status, 0, sizeof(DevStatus), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(S->blk_idx, 0xff, sizeof(int) * nb, st);
    // look-back status words: this sub-batch's epochs are new, but the inverse
    // reuses the memory, and a word it left could carry one of them
    const size_t big_tiles = (size_t)N / 2048 + (size_t)N / 4097 + 4;
    if (e == cudaSuccess) e = cudaMemsetAsync(f.status64, 0, sizeof(unsigned long long) * 256 * big_tiles, st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(f.split_status, 0, sizeof(unsigned long long) * 4 * ((size_t)N / kWT + 2), st);
    if (e != cudaSuccess) return map_cuda_error(e);

    // ---- alphabet, initial keys
    int ntiles = (int)tiles.size();
    QZ_LAUNCH(S, st, "k_block_hist", N,
              k_block_hist<<<grid_for(ntiles, 4, S->sms * 8), kThreads, 0, st>>>(d_T, S->tiles, ntiles, S->blk_off,
                                                                                S->blk_hist));
    QZ_LAUNCH(S, st, "k_block_alpha", 1280ll * nb,
              k_block_alpha<<<nb, kThreads, 0, st>>>(S->blk_hist, S->blk_code, S->blk_K, S->blk_sigma));
    // reads T once, writes key, R (the same text key, in text order), W and G
    QZ_LAUNCH(S, st, "k_init_keys", 17 * N,
              k_init_keys<<<ntiles, kThreads, 0, st>>>(d_T, S->tiles, S->blk_off, S->blk_code, S->blk_K,
                                                       S->blk_sigma, f.key, f.W[0], f.G[0],
                                                       reinterpret_cast<uint32_t*>(f.R)));
    // suffix-array entries not set by the initial split stay -1 for the fixup
    e = cudaMemsetAsync(f.SA, 0xff, sizeof(int) * N, st);
    if (e != cudaSuccess) return map_cuda_error(e);
    const bool dump = dump_on() && N <= (1 << 20);
    if (dump) {
        dump_array("init_key", f.key, 4 * N, st);
        dump_array("init_W", f.W[0], 4 * N, st);
        dump_array("init_G", f.G[0], 4 * N, st);
    }
    int cur = 0;
    int act = CNT_ACTIVE;  // counter slot holding the current active count
    // ---- initial sort (groups = blocks)
    // initial keys: up to 32 bits of packed symbols
    sort_groups(S, cnt0, (int)N, S->counters + act, f.key, f.W[0], f.G[0], st, false, 32);
    if (dump) {
        dump_array("sorted_key", f.key, 4 * N, st);
        dump_array("sorted_W", f.W[0], 4 * N, st);
    }
    auto split = [&](long long A, int rank_mode) {
        SplitArgs a;
        a.A = S->counters + act;
        a.A_next = S->counters + (act ^ (CNT_ACTIVE ^ CNT_ACTIVE_ALT));
        a.key = f.key;
        a.G = f.G[cur];
        a.W = f.W[cur];
        a.R = f.R;
        a.SA = f.SA;
        a.Wn = f.W[cur ^ 1];
        a.Gn = f.G[cur ^ 1];
        a.list_rbc = f.list_rbc;
        a.list_med = f.list_med;
        a.list_tile = f.list_tile;
        a.list_large = f.list_large;
        a.counters = S->counters;
        a.p_surv = f.p_surv;
        a.p_sub = f.p_sub;
        a.p_grp = f.p_grp;
        a.write_rank = rank_mode;
        a.medium_max = S->tune.medium_max;
        a.n = (int)N;
        a.st = S->status;
        long long tiles_n = (A + kWT - 1) / kWT;
        // the class counters the split appends to (and its ticket) start at zero
        if (!S->dry && e == cudaSuccess)
            e = cudaMemsetAsync(S->counters + CNT_SPLIT_FIRST, 0, sizeof(int) * (CNT_SPLIT_END - CNT_SPLIT_FIRST), st);
        if (S->tune.split_lookback) {
            // key, group rank and suffix of every slot in; 24 bytes of status
            // per tile out; the rest is added once the survivors are known
            unsigned epoch = ++S->radix_epoch & 0x3fffffffu;
            if (epoch == 0) epoch = ++S->radix_epoch & 0x3fffffffu;
            const bool test = S->tune.lookback_test == 2;
            SplitLookBack lb{f.split_status, reinterpret_cast<unsigned*>(S->counters + CNT_SPLIT_TICKET), epoch,
                             test ? 4096u : kSplitSpinLimit, test ? 1 : -1};
            const long long ctiles = (A + kCT - 1) / kCT;
            const int grid = (int)std::max(1ll, std::min<long long>(ctiles, (long long)S->sms * 5));
            QZ_LAUNCH(S, st, rank_mode == kRankNone ? "k_split_first" : "k_split", 12 * A + 24 * ctiles,
                      k_split<<<grid, kThreads, 0, st>>>(a, lb));
            cur ^= 1;
            act ^= CNT_ACTIVE ^ CNT_ACTIVE_ALT;
            return;
        }
        int grid = grid_for((A + kWT - 1) / kWT, kWarps, S->sms * 8);
        // count: key and group rank of every slot; 12 bytes of partials per tile
        QZ_LAUNCH(S, st, "k_split_count", 8 * A + 12 * tiles_n, k_split_count<<<grid, kThreads, 0, st>>>(a));
        if (tiles_n <= kPscanSingleMax) {
            QZ_LAUNCH(S, st, "k_pscan_single", 24 * tiles_n, k_pscan_single<<<1, kThreads, 0, st>>>(a));
        } else {
            QZ_LAUNCH(S, st, "k_pscan_reduce", 12 * tiles_n,
                      k_pscan_reduce<<<kScanGrid, kThreads, 0, st>>>(a, f.c_surv, f.c_sub, f.c_grp));
            QZ_LAUNCH(S, st, "k_pscan_top", 24ll * kScanGrid,
                      k_pscan_top<<<1, kThreads, 0, st>>>(a, f.c_surv, f.c_sub, f.c_grp, kScanGrid));
            QZ_LAUNCH(S, st, "k_pscan_apply", 24 * tiles_n,
                      k_pscan_apply<<<kScanGrid, kThreads, 0, st>>>(a, f.c_surv, f.c_sub, f.c_grp));
        }
        // apply: key, group, suffix in; ranks out per rank_mode; then the
        // suffix either leaves (SA) or is compacted (2 words); fixed up below
        QZ_LAUNCH(S, st, rank_mode == kRankNone ? "k_split_apply_first" : "k_split_apply", 12 * A + 12 * tiles_n,
                  k_split_apply<<<grid, kThreads, 0, st>>>(a));
        cur ^= 1;
        act ^= CNT_ACTIVE ^ CNT_ACTIVE_ALT;
    };
    auto dump_split = [&]() {
        if (!dump) return;
        dump_array("split_counters", S->counters, 4 * CNT_SLOTS, st);
        dump_array("split_R", f.R, 4 * N, st);
        dump_array("split_SA", f.SA, 4 * N, st);
        dump_array("split_W", f.W[cur], 4 * N, st);
        dump_array("split_G", f.G[cur], 4 * N, st);
    };
    split(N, kRankNone);
    dump_split();
    add_round(S, 0, N);

    // rank keys R[x+h] + h + 1 (R < N, h <= n_b) and end keys (<= n_b): below N + max n_b
    int nmax = 0;
    for (int b = 0; b < nb; ++b) nmax = std::max(nmax, n[b]);
    int rank_key_bits = 1;
    while (rank_key_bits < 32 && (1ll << rank_key_bits) <= N + nmax) ++rank_key_bits;
    bool fixed_up = false;
    auto rank_fixup = [&](long long finished) {
        // SA read; one rank written per suffix the initial split finished
        QZ_LAUNCH(S, st, "k_rank_fixup", 4 * N + 4 * finished,
                  k_rank_fixup<<<grid_for(N, kThreads, S->sms * 16), kThreads, 0, st>>>((int)N, f.SA, f.R));
        fixed_up = true;
    };
    GatherArgs ga{f.R, S->blk_off, nb, S->blk_K, 0};
    // One doubling round on the device.  hc: the round's list counts (exact,
    // or bounds when the round is issued ahead of its counts); A: its active
    // slots (or a bound).  Every kernel reads the exact counts from the device.
    auto issue_round = [&](int r, const int* hc, long long A) {
        ga.round = r;
        // suffix and group rank read, one rank gathered, key written; small
        // groups inside a warp window sorted on the spot (suffix rewritten)
        const long long small_el = A - hc[CNT_PAIR_ELEMS] - hc[CNT_MED_ELEMS] - hc[CNT_TILE_ELEMS] -
                                   hc[CNT_LARGE_ELEMS];
        QZ_LAUNCH(S, st, "k_gather_small", 16ll * A + 4ll * std::max(small_el, 0ll),
                  k_gather_small<<<grid_for(((A + 31) / 32 + kGatherRun - 1) / kGatherRun, kWarps, S->sms * 16),
                                   kThreads, 0, st>>>(S->counters + act, f.G[cur], f.key, f.W[cur], ga, f.straddle));
        if (r == 0) rank_fixup(N - A);
        // one flag byte per gather run; flagged runs: group ranks of one window,
        // keys and suffixes of the straddling group
        const long long nruns = ((A + 31) / 32 + kGatherRun - 1) / kGatherRun;
        QZ_LAUNCH(S, st, "k_sort_straddle", nruns,
                  k_sort_straddle<<<grid_for(nruns, kWarps, S->sms * 16), kThreads, 0, st>>>(
                      S->counters + act, f.G[cur], f.key, f.W[cur], f.straddle));
        // round 0 gathers 32-bit text keys; later rounds rank keys below N + max n_b
        sort_groups(S, hc, (int)A, S->counters + act, f.key, f.W[cur], f.G[cur], st, true,
                    r == 0 ? 32 : rank_key_bits);
        if (dump && !S->dry) {
            dump_array("rsorted_key", f.key, 4 * (size_t)A, st);
            dump_array("rsorted_W", f.W[cur], 4 * (size_t)A, st);
        }
        split(A, r == 0 ? kRankAll : kRankChanged);
        if (!S->dry) dump_split();
    };

    // ---- doubling rounds.  Host-paced (default): the counters of the split
    // that lists a round's groups are read back, then the round is issued with
    // launch shapes from its exact counts.  Pipelined (tune.round_pipeline):
    // round r is issued before those counters are read, so the device always
    // has the next round queued; its launch shapes come from bounds (active
    // counts and group lengths only shrink from round to round, so the
    // previous round's counts bound this one's) and the round after the last
    // finds no active slot and returns at once.  It saves the host read's
    // bubble per round and costs launches sized for bounds plus one empty
    // round.  Counters and status of each split land in one of two pinned
    // slots.
    int* hc[2] = {S->pin_rd, S->pin_rd + CNT_SLOTS};
    DevStatus* hs[2] = {reinterpret_cast<DevStatus*>(S->pin_rd + S->cap_blocks + 64),
                        reinterpret_cast<DevStatus*>(S->pin_rd + S->cap_blocks + 68)};
    auto post = [&](int slot) {
        if (e == cudaSuccess) e = cudaMemcpyAsync(hc[slot], S->counters, sizeof(int) * CNT_SLOTS, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(hs[slot], S->status, sizeof(DevStatus), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaEventRecord(S->round_ev[slot], st);
    };
    // largest class with a listed group: a round's groups lie inside the
    // previous round's, so no later round has a longer one
    auto top_class = [](const int* h) {
        return h[CNT_LARGE] ? 4 : h[CNT_TILE] ? 3 : h[CNT_MED] ? 2 : h[CNT_PAIR] ? 1 : 0;
    };
    auto bounds = [&](int top, long long A, int* out) {
        for (int i = 0; i < CNT_SLOTS; ++i) out[i] = 0;
        const int lo[5] = {0, kSmallMax + 1, 65, S->tune.medium_max + 1, kOT + 1};
        const int cnt[5] = {0, CNT_PAIR, CNT_MED, CNT_TILE, CNT_LARGE};
        const int el[5] = {0, CNT_PAIR_ELEMS, CNT_MED_ELEMS, CNT_TILE_ELEMS, CNT_LARGE_ELEMS};
        for (int c = 1; c <= top; ++c) {
            out[cnt[c]] = (int)std::max<long long>(1, A / lo[c]);
            out[el[c]] = (int)A;
        }
    };
    post(0);  // lists of round 0, from the initial split
    if (e != cudaSuccess) return map_cuda_error(e);
    int top = top_class(cnt0);  // the initial groups are the blocks
    long long A_bound = N, A_prev = N;
    int round = 0;
    // profile record of the previous round's split apply (its survivors are
    // known one round later)
    int last_apply = -1;
    if (S->profile && !S->prof_pending.empty() && split_store_kernel(S->prof_pending.back().name))
        last_apply = (int)S->prof_pending.size() - 1;
    int hb[CNT_SLOTS];
    for (;;) {
        if (round >= kMaxRounds) {
            if (debug_on()) debug_log("no convergence after %d rounds", round);
            cudaStreamSynchronize(st);
            prof_flush(S);
            return QZGPU_GPU_ERROR;
        }
        const int act_r = act;  // this round's active count lives here
        const size_t mark = S->prof_pending.size();
        if (S->tune.round_pipeline) {
            bounds(top, A_bound, hb);
            issue_round(round, hb, A_bound);
            post((round + 1) & 1);
        }
        if (e == cudaSuccess) e = cudaEventSynchronize(S->round_ev[round & 1]);
        if (e != cudaSuccess) return map_cuda_error(e);
        if (hs[round & 1]->error) {
            // the counters of a round that failed are not to be trusted
            const DevStatus ds = *hs[round & 1];
            cudaStreamSynchronize(st);
            prof_flush(S);
            if (debug_on()) debug_log("device status %d at %d detail %lld", ds.error, ds.where, ds.detail);
            return ds.error;
        }
        const int* h = hc[round & 1];
        const int A = h[act_r];
        if (!S->tune.round_pipeline) {
            // host-paced: the round is issued with its exact counts, after they
            // are read; its launches carry exact bytes
            if (S->profile && last_apply >= 0)
                S->prof_pending[last_apply].bytes +=
                    8ll * A + 4ll * (A_prev - A) + (round == 1 ? 4ll * A_prev : 0);
            if (A == 0) break;
            if (debug_on())
                debug_log("round %d: active %d rbc %d/%d medium %d/%d tile %d/%d large %d/%d", round, A, h[CNT_PAIR],
                          h[CNT_PAIR_ELEMS], h[CNT_MED], h[CNT_MED_ELEMS], h[CNT_TILE], h[CNT_TILE_ELEMS],
                          h[CNT_LARGE], h[CNT_LARGE_ELEMS]);
            add_round(S, round + 1, A);
            std::copy(h, h + CNT_SLOTS, hb);  // the pinned slot is rewritten by the next post
            issue_round(round, hb, A);
            post((round + 1) & 1);
            last_apply = -1;
            if (S->profile && !S->prof_pending.empty() && split_store_kernel(S->prof_pending.back().name))
                last_apply = (int)S->prof_pending.size() - 1;
            A_prev = A;
            ++round;
            continue;
        }
        if (S->profile) {
            // the previous split wrote A survivors (8 B) and A_prev - A
            // suffix-array entries (4 B), and round 0's split 4 B of rank per slot
            if (last_apply >= 0)
                S->prof_pending[last_apply].bytes +=
                    8ll * A + 4ll * (A_prev - A) + (round == 1 ? 4ll * A_prev : 0);
            // this round's launches, bytes recomputed from its exact counts
            // (a launch the exact counts would not make did no work)
            const bool fu = fixed_up;
            const int c0 = cur, a0 = act;
            const unsigned ep = S->radix_epoch;
            cur = c0 ^ 1;  // the state this round was issued in
            act = act_r;
            S->dry = true;
            S->dry_list.clear();
            issue_round(round, h, A);
            S->dry = false;
            cur = c0;
            act = a0;
            fixed_up = fu;
            S->radix_epoch = ep;
            // records in issue order (only some kernels may be timed): each
            // takes the next dry launch of its name
            size_t k = 0;
            last_apply = -1;
            for (size_t i = mark; i < S->prof_pending.size(); ++i) {
                auto& rec = S->prof_pending[i];
                size_t j = k;
                while (j < S->dry_list.size() && strcmp(S->dry_list[j].first, rec.name) != 0) ++j;
                if (j < S->dry_list.size()) {
                    rec.bytes = S->dry_list[j].second;
                    k = j + 1;
                } else {
                    rec.bytes = 0;
                }
                if (split_store_kernel(rec.name)) last_apply = (int)i;
            }
        }
        if (A == 0) break;  // the round just issued finds nothing to do
        if (debug_on())
            debug_log("round %d: active %d rbc %d/%d medium %d/%d tile %d/%d large %d/%d", round, A, h[CNT_PAIR],
                      h[CNT_PAIR_ELEMS], h[CNT_MED], h[CNT_MED_ELEMS], h[CNT_TILE], h[CNT_TILE_ELEMS], h[CNT_LARGE],
                      h[CNT_LARGE_ELEMS]);
        add_round(S, round + 1, A);
        A_prev = A;
        A_bound = A;
        top = top_class(h);
        ++round;
    }
    if (!fixed_up) rank_fixup(N);  // the initial sort finished every suffix

    // ---- U and primary indexes: SA read, one byte gathered, one written
    int* hcnt = S->pin_rd;
    DevStatus& hst = *hs[0];
    QZ_LAUNCH(S, st, "k_extract", 6 * N,
              k_extract<<<grid_for(N, kThreads, S->sms * 16), kThreads, 0, st>>>(
                  (int)N, f.SA, f.R, d_T, S->blk_off, nb, d_U, S->blk_idx, aux_rate ? S->blk_aux_rate : nullptr,
                  S->blk_aux_off, S->aux, S->status));
    e = cudaMemcpyAsync(hcnt, S->blk_idx, sizeof(int) * nb, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hst, S->status, sizeof(hst), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && aux_out && aux_total)
        e = cudaMemcpyAsync(aux_out, S->aux, sizeof(int) * aux_total, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return map_cuda_error(e);
    prof_flush(S);
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
    *rounds_out = round;
    return QZGPU_NO_ERROR;
}

}  // namespace

// Batches are processed in sub-batches of at most kSubBatchBytes (a larger
// block alone): the random rank gathers and scatters of a round then stay
// within one sub-batch's rank array, which the 126 MB L2 largely holds.
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
    S->launches = 0;
    int max_rounds = 0;
    long long off = 0;
    int aoff = 0;
    for (int b0 = 0; b0 < nb;) {
        int b1 = b0;
        long long sub = 0;
        while (b1 < nb && (b1 == b0 || sub + n[b1] <= S->sub_batch_bytes)) sub += n[b1++];
        int rounds = 0;
        int rc = forward_core(S, b1 - b0, n + b0, d_T + off, d_U + off, idx + b0, aux_rate ? aux_rate + b0 : nullptr,
                              aux_out ? aux_out + aoff : nullptr, st, &rounds);
        if (rc) return rc;
        if (aux_rate)
            for (int b = b0; b < b1; ++b)
                if (aux_rate[b] > 0 && n[b] > 0) aoff += (n[b] - 1) / aux_rate[b];
        if (rounds > max_rounds) max_rounds = rounds;
        off += sub;
        b0 = b1;
    }
    long long active_sum = 0;
    for (long long a : S->rounds_active) active_sum += a;
    S->stats.rounds = max_rounds;
    S->stats.kernel_launches = S->launches;
    S->stats.active_total = active_sum;
    S->stats.alg_bytes = 15 * N + 28 * active_sum;
    return QZGPU_NO_ERROR;
}

}  // namespace qz
