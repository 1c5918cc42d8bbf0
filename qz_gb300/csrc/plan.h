// Sub-batch plan of a batched call (plain C++, no device code): which
// consecutive blocks each lane job covers and the order lanes take the jobs.
#pragma once
#include <algorithm>
#include <vector>

namespace qz {

struct SubBatch {
    int b0, b1;            // blocks [b0, b1)
    long long off, bytes;  // byte offset of block b0 in the batch, bytes covered
    int seq;               // place in the order the lanes take sub-batches
};

// Cuts nb blocks of sizes n[] into sub-batches of consecutive whole blocks of
// at most `limit` bytes (a block larger than `limit` alone).  Sub-batches
// above `lane_bytes` go to `big`: only the full-capacity lane can hold them,
// and it runs them first.  The others go to `small`, largest first
// (longest-processing-time order, bytes standing for time), so that no large
// sub-batch starts last and runs alone while the other lanes idle.  seq
// numbers big then small.  Blocks keep their places in the input and output
// buffers; only the order of work changes.
inline void plan_sub_batches(int nb, const int* n, long long limit, long long lane_bytes,
                             std::vector<SubBatch>* big, std::vector<SubBatch>* small) {
    big->clear();
    small->clear();
    long long off = 0;
    for (int b0 = 0; b0 < nb;) {
        int b1 = b0;
        long long bytes = 0;
        while (b1 < nb && (b1 == b0 || bytes + n[b1] <= limit)) bytes += n[b1++];
        (bytes > lane_bytes ? big : small)->push_back(SubBatch{b0, b1, off, bytes, 0});
        off += bytes;
        b0 = b1;
    }
    std::stable_sort(small->begin(), small->end(),
                     [](const SubBatch& x, const SubBatch& y) { return x.bytes > y.bytes; });
    int seq = 0;
    for (SubBatch& sb : *big) sb.seq = seq++;
    for (SubBatch& sb : *small) sb.seq = seq++;
}

}  // namespace qz
