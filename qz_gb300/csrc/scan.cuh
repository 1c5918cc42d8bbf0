// Device-wide exclusive prefix sum of uint32 counts (reduce-then-scan).
// The length may live in device memory, so the three launches have fixed
// shapes and can be issued without a host round trip.
#pragma once
#include "common.cuh"

namespace qz {

constexpr int kScanGrid = 256;              // CTAs in the reduce/apply phases
constexpr int kScanItems = 4;               // uint32 per thread per tile (one uint4)
constexpr int kScanTile = kThreads * kScanItems;

struct Storage;
// `len_dev` (if not null) overrides `len`.  Uses S->partial as scratch.
void scan_exclusive(Storage* S, const uint32_t* in, uint32_t* out, int len, const int* len_dev,
                    uint32_t* total_dev, cudaStream_t st);

}  // namespace qz
