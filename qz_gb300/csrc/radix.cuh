// Segmented (key, value) sorts for groups longer than a warp sorts.
#pragma once
#include "engine.h"

namespace qz {

struct BigArgs {
    const int2* list;        // (first slot, length) per group
    const int* nseg;         // number of groups (device)
    const uint32_t* tbase;   // first tile of each group
    const uint32_t* wbase;   // first workspace slot of each group
    const int* ntiles;       // total tiles (device)
    uint32_t* gmask;         // per group: passes whose digit is not constant (bit p)
    uint32_t* tseg;          // group of each tile (written by the histogram kernel)
    int4* tdesc;             // per tile, written by pass 0 for the stable passes:
    int2* tdesc2;            //   (group, pass mask, first slot, workspace base), (tile in group, length)
};

// Where a group's slots are before / after one of its needed passes: the first
// needed pass reads the compact (key, val) arrays, the last writes them back,
// the others ping-pong through the two workspaces.
struct BigBuffers {
    uint32_t* key;
    int* val;
    uint32_t* wsk[2];
    int* wsv[2];
};

// Listed groups sorted by key: read from (skey, sval) and written to (key,
// val) at the same slots (the two may be the same arrays).  host_count and
// elems are host copies (or bounds) of the group and slot counts; d_count is
// the device count the kernels read.
// Groups of medium_max+1 .. kOT slots (one CTA each, all passes in shared memory).
// key_bits: the keys are below 2^key_bits (sets the first digit's width, as
// for the large groups).
void sort_tile_groups(Storage* S, const int2* list, const int* d_count, int host_count, long long elems,
                      const uint32_t* skey, const int* sval, uint32_t* key, int* val, int key_bits,
                      cudaStream_t st);
// Groups of 17..64 slots (one warp each, rank by count; fwd.cu).
void sort_rbc_groups(Storage* S, const int2* list, const int* d_count, int host_count, long long elems,
                     const uint32_t* skey, const int* sval, uint32_t* key, int* val, cudaStream_t st);
// Groups of 65..medium_max slots (one warp each, LSD radix in shared memory; fwd.cu).
void sort_medium_groups(Storage* S, const int2* list, const int* d_count, int host_count, long long elems,
                        const uint32_t* skey, const int* sval, uint32_t* key, int* val, cudaStream_t st);
// Groups longer than kOT slots, in place in (key, val) (one decoupled
// look-back pass per digit).  key_bits: the keys are below 2^key_bits, which
// sets the digit layout (three passes up to 16 + the tuned first-digit width).
void sort_big_groups(Storage* S, const int2* list, const int* d_count, int host_count, long long elems,
                     uint32_t* key, int* val, int key_bits, cudaStream_t st);
size_t tile_sort_smem();
// Digit-count words per listed group of the large-group sort.
size_t big_hist_words();

}  // namespace qz
