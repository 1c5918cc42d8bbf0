// Shared device helpers for the block-sorting kernels (sm_103a).
// Integer-only code: warp shuffles and shared-memory scans, no tensor cores.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/qzgpu.h"

namespace qz {

constexpr int kThreads = 256;  // threads per CTA for the streaming kernels
constexpr int kWarps = kThreads / 32;

// Device status word: kernels never trap; they record the first problem here
// and return, and the host turns it into a QZGPU_* error code.
struct DevStatus {
    int error;   // QZGPU_* code, 0 if fine
    int where;   // kernel tag
    long long detail;
};

__device__ __forceinline__ void report(DevStatus* st, int code, int where, long long detail) {
    if (atomicCAS(&st->error, 0, code) == 0) {
        st->where = where;
        st->detail = detail;
    }
}

// A problem that belongs to one block of a batch (an inverse BWT that cannot
// be inverted): recorded for that block as well, so that a caller batching
// independent requests can fail the one request and keep the others.
__device__ __forceinline__ void report_block(DevStatus* st, int* blk_status, int code, int where, int b) {
    if (blk_status) atomicCAS(blk_status + b, 0, code);
    report(st, code, where, b);
}

// True once any kernel has reported a problem: the kernels whose stores are
// addressed by data that an earlier failure may have left inconsistent (suffix
// indexes, digit positions) return at entry instead.
__device__ __forceinline__ bool failed(const DevStatus* st) {
    return *reinterpret_cast<const volatile int*>(&st->error) != 0;
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned warp_id() { return threadIdx.x >> 5; }

template <typename T>
__device__ __forceinline__ T warp_incl_sum(T v) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T t = __shfl_up_sync(0xffffffffu, v, d);
        if ((int)lane_id() >= d) v += t;
    }
    return v;
}

__device__ __forceinline__ int warp_incl_max(int v) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, d);
        if ((int)lane_id() >= d) v = max(v, t);
    }
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    return v;
}

// 4-byte asynchronous copy global -> shared memory.  The copy is visible to
// the issuing thread after cp_async_wait_all(); other threads need a barrier
// after that wait as well.
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Bulk copies (the asynchronous copy unit, 1-D form) into this CTA's shared
// memory, completed on an mbarrier: both addresses 16-byte aligned and the
// size a multiple of 16 bytes.  A CTA launched without a cluster is a cluster
// of one, so its own shared addresses serve as shared::cluster addresses.
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes the initialised barriers visible to the asynchronous copy unit (then a
// CTA barrier before any thread uses them).
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Waits for the phase with the given parity to complete, at most `limit`
// polls; false if the limit ran out.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, unsigned limit) {
    const unsigned a = smem_u32(bar);
    for (unsigned i = 0; i < limit; ++i) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Orders this thread's earlier shared-memory accesses (and, after a CTA
// barrier, the other threads') before later bulk copies into the same bytes.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void bulk_g2s(void* smem_dst, const void* gmem_src, unsigned bytes,
                                         unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(smem_dst)),
        "l"(gmem_src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Stable rank of this lane's item among the lanes of its warp that hold the
// same digit, plus the running count of that digit (per-warp counters `cnt`,
// one per digit): returns the count before this warp step plus the lanes with
// the same digit below this one, and advances the count.  Invalid lanes take
// no part.
//
// RANK picks how the lanes with the same 8-bit digit are found:
//   0: one warp match instruction;
//   1: eight ballots, one per digit bit (integer pipes, no match);
//   2: a match on the high four bits and four ballots on the low four.
template <int RANK = 0>
__device__ __forceinline__ unsigned warp_digit_peers(unsigned dg, bool valid) {
    if (RANK == 0) return __match_any_sync(0xffffffffu, valid ? dg : 0x10000u);
    constexpr int LOW = RANK == 1 ? 8 : 4;
    unsigned peers = RANK == 1 ? __ballot_sync(0xffffffffu, valid)
                               : __match_any_sync(0xffffffffu, valid ? (dg >> 4) : 0x10000u);
#pragma unroll
    for (int b = 0; b < LOW; ++b) {
        const unsigned bit = (dg >> b) & 1u;
        const unsigned m = __ballot_sync(0xffffffffu, bit);
        peers &= m ^ (bit - 1u);  // m where the bit is set, ~m where it is clear
    }
    return peers;
}

template <int RANK = 0>
__device__ __forceinline__ uint32_t warp_digit_rank(unsigned dg, bool valid, uint32_t* cnt) {
    const unsigned lt = (1u << lane_id()) - 1u;
    const unsigned peers = warp_digit_peers<RANK>(dg, valid);
    const unsigned before = __popc(peers & lt);
    const uint32_t prev = valid ? cnt[dg] : 0u;
    __syncwarp();
    if (valid && before == 0) cnt[dg] = prev + __popc(peers);
    __syncwarp();
    return prev + before;
}

// Block-wide exclusive sum over kThreads threads. `sh` needs kWarps+1 slots.
// Returns the exclusive prefix for this thread; *total receives the sum.
template <typename T>
__device__ __forceinline__ T block_excl_sum(T v, T* sh, T* total) {
    T inc = warp_incl_sum(v);
    if (lane_id() == 31) sh[warp_id()] = inc;
    __syncthreads();
    if (warp_id() == 0) {
        T w = lane_id() < (unsigned)kWarps ? sh[lane_id()] : T(0);
        T wi = warp_incl_sum(w);
        if (lane_id() < (unsigned)kWarps) sh[lane_id()] = wi - w;
        if (lane_id() == (unsigned)kWarps - 1) sh[kWarps] = wi;
    }
    __syncthreads();
    T res = sh[warp_id()] + inc - v;
    *total = sh[kWarps];
    __syncthreads();
    return res;
}

// Block-wide inclusive max over kThreads threads. `sh` needs kWarps+1 slots.
__device__ __forceinline__ int block_incl_max(int v, int* sh, int* total) {
    int inc = warp_incl_max(v);
    if (lane_id() == 31) sh[warp_id()] = inc;
    __syncthreads();
    if (warp_id() == 0) {
        int w = lane_id() < (unsigned)kWarps ? sh[lane_id()] : INT32_MIN;
        int wi = warp_incl_max(w);
        int ex = __shfl_up_sync(0xffffffffu, wi, 1);
        if (lane_id() == 0) ex = INT32_MIN;
        if (lane_id() < (unsigned)kWarps) sh[lane_id()] = ex;
        if (lane_id() == (unsigned)kWarps - 1) sh[kWarps] = wi;
    }
    __syncthreads();
    int res = max(sh[warp_id()], inc);
    *total = sh[kWarps];
    __syncthreads();
    return res;
}

// Rank-array accesses with an L2 evict-last policy: the random rank gathers and
// scatters of a round reuse the same array, while the slot arrays stream
// through with evict-first hints.
__device__ __forceinline__ unsigned long long l2_keep_policy() {
    unsigned long long pol;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

__device__ __forceinline__ int ld_keep(const int* p, unsigned long long pol) {
    int v;
    asm volatile("ld.global.nc.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
    return v;
}

__device__ __forceinline__ void st_keep(int* p, int v, unsigned long long pol) {
    asm volatile("st.global.L2::cache_hint.b32 [%0], %1, %2;" ::"l"(p), "r"(v), "l"(pol) : "memory");
}

// Index of the block that owns global position x: off[b] <= x < off[b+1].
__device__ __forceinline__ int block_of(const int* __restrict__ off, int nblocks, int x) {
    int lo = 0, hi = nblocks - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= x) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Chunk of [0, len) owned by CTA `c` of `grid`, rounded to `align` elements.
__device__ __forceinline__ void chunk_range(int len, int grid, int c, int align, int* lo, int* hi) {
    long long per = ((long long)len + grid - 1) / grid;
    per = (per + align - 1) / align * align;
    long long a = per * c, b = a + per;
    if (a > len) a = len;
    if (b > len) b = len;
    *lo = (int)a;
    *hi = (int)b;
}

}  // namespace qz
