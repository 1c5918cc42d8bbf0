#include "scan.cuh"
#include "engine.h"

namespace qz {

__device__ __forceinline__ int resolve_len(int len, const int* len_dev) { return len_dev ? *len_dev : len; }

// Loads four consecutive counts starting at k (k is a multiple of 4).
__device__ __forceinline__ uint4 load4(const uint32_t* in, int k, int len) {
    if (k + 3 < len) return *reinterpret_cast<const uint4*>(in + k);
    uint4 v = make_uint4(0, 0, 0, 0);
    if (k < len) v.x = in[k];
    if (k + 1 < len) v.y = in[k + 1];
    if (k + 2 < len) v.z = in[k + 2];
    return v;
}

__global__ void __launch_bounds__(kThreads) k_scan_reduce(const uint32_t* __restrict__ in, int len_h,
                                                          const int* __restrict__ len_dev,
                                                          uint32_t* __restrict__ partial) {
    __shared__ uint32_t sh[kWarps + 1];
    int len = resolve_len(len_h, len_dev);
    int lo, hi;
    chunk_range(len, gridDim.x, blockIdx.x, kScanTile, &lo, &hi);
    uint32_t acc = 0;
    for (int base = lo; base < hi; base += kScanTile) {
        int k = base + threadIdx.x * kScanItems;
        uint4 v = load4(in, k, hi);
        acc += v.x + v.y + v.z + v.w;
    }
    uint32_t tot;
    block_excl_sum(acc, sh, &tot);
    if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

// One CTA: exclusive scan of the per-CTA partials in place; writes the total.
__global__ void __launch_bounds__(kThreads) k_scan_top(uint32_t* __restrict__ partial, int n,
                                                       uint32_t* __restrict__ total_dev) {
    __shared__ uint32_t sh[kWarps + 1];
    uint32_t carry = 0;
    for (int base = 0; base < n; base += kThreads) {
        int i = base + threadIdx.x;
        uint32_t v = i < n ? partial[i] : 0;
        uint32_t tot;
        uint32_t ex = block_excl_sum(v, sh, &tot);
        if (i < n) partial[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0 && total_dev) *total_dev = carry;
}

__global__ void __launch_bounds__(kThreads) k_scan_apply(const uint32_t* in,
                                                         uint32_t* out, int len_h,
                                                         const int* __restrict__ len_dev,
                                                         const uint32_t* __restrict__ partial) {
    __shared__ uint32_t sh[kWarps + 1];
    int len = resolve_len(len_h, len_dev);
    int lo, hi;
    chunk_range(len, gridDim.x, blockIdx.x, kScanTile, &lo, &hi);
    uint32_t carry = partial[blockIdx.x];
    for (int base = lo; base < hi; base += kScanTile) {
        int k = base + threadIdx.x * kScanItems;
        uint4 v = load4(in, k, hi);
        uint32_t s = v.x + v.y + v.z + v.w;
        uint32_t tot;
        uint32_t ex = block_excl_sum(s, sh, &tot) + carry;
        uint4 o;
        o.x = ex;
        o.y = ex + v.x;
        o.z = o.y + v.y;
        o.w = o.z + v.z;
        if (k + 3 < hi) {
            *reinterpret_cast<uint4*>(out + k) = o;
        } else {
            if (k < hi) out[k] = o.x;
            if (k + 1 < hi) out[k + 1] = o.y;
            if (k + 2 < hi) out[k + 2] = o.z;
        }
        carry += tot;
    }
}

void scan_exclusive(Storage* S, const uint32_t* in, uint32_t* out, int len, const int* len_dev,
                    uint32_t* total_dev, cudaStream_t st) {
    uint32_t* partial = S->partial;
    // bytes assume the host length; device-sized scans report 0
    long long b = len_dev ? 0 : 12ll * len;
    QZ_LAUNCH(S, st, "k_scan_reduce", b / 3,
              k_scan_reduce<<<kScanGrid, kThreads, 0, st>>>(in, len, len_dev, partial));
    QZ_LAUNCH(S, st, "k_scan_top", 8 * kScanGrid, k_scan_top<<<1, kThreads, 0, st>>>(partial, kScanGrid, total_dev));
    QZ_LAUNCH(S, st, "k_scan_apply", 2 * b / 3,
              k_scan_apply<<<kScanGrid, kThreads, 0, st>>>(in, out, len, len_dev, partial));
}

}  // namespace qz
