// Batched calls on a multi-lane engine.
//
// A storage handed to callers (qzgpu_storage) is an engine of K lanes (three
// by default: measured best on a 33-block chunk and on 256 uneven blocks;
// QZGPU_LANES overrides).  Each
// lane is a full scratch set (Storage) with its own stream and a persistent
// worker thread.  A batch is cut into sub-batches of at most lane_bytes block
// bytes (blocks kept whole); lanes take sub-batches, largest first, as they
// become free, so the latency-bound phases of one sub-batch (dependent
// gathers, per-round host reads of the counters) overlap with the work of the
// others on the device.
// Lane 0 is sized for the whole capacity and alone takes a block larger than
// lane_bytes.
#include <algorithm>
#include <atomic>
#include <cstdlib>

#include "engine.h"
#include "plan.h"

namespace qz {

namespace {

constexpr long long kTouchMinBytes = 8ll << 20;  // smaller host batches copy out directly

// True when every output buffer is page-locked host memory (cudaMallocHost,
// cudaHostAlloc or cudaHostRegister): its pages are resident, so copies into
// it need no touching first.
bool outputs_pinned(int nb, const int* n, unsigned char* const* hout) {
    for (int b = 0; b < nb; ++b) {
        if (n[b] <= 0) continue;
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, hout[b]) != cudaSuccess) {
            cudaGetLastError();  // clear it: the pointer is plain pageable memory
            return false;
        }
        if (at.type != cudaMemoryTypeHost) return false;
    }
    return true;
}

int lanes_for(long long cap_bytes) {
    const char* env = getenv("QZGPU_LANES");
    if (env && atoi(env) > 0) return std::min(atoi(env), 16);
    return cap_bytes > kLaneBytes ? 3 : 1;
}

}  // namespace

size_t engine_device_bytes(long long cap_bytes, int cap_blocks) {
    int k = lanes_for(cap_bytes);
    size_t b = storage_device_bytes(cap_bytes, cap_blocks);
    if (k > 1) b += (size_t)(k - 1) * storage_device_bytes(std::min(cap_bytes, kLaneBytes), cap_blocks);
    return b;
}

int engine_init(Engine* E, long long cap_bytes, int cap_blocks) {
    E->cap_bytes = cap_bytes;
    E->cap_blocks = cap_blocks;
    E->lane_bytes = std::min(cap_bytes, kLaneBytes);
    int k = lanes_for(cap_bytes);
    for (int i = 0; i < k; ++i) {
        auto s = std::make_unique<Storage>();
        int rc = storage_init(s.get(), i == 0 ? cap_bytes : E->lane_bytes, cap_blocks);
        if (rc) {
            engine_free(E);
            return rc;
        }
        E->lanes.push_back(std::move(s));
    }
    E->device = E->lanes[0]->device;
    for (int i = 0; i < k; ++i) {
        E->threads.emplace_back([E, i] {
            cudaSetDevice(E->device);
            int seen = 0;
            for (;;) {
                std::function<void(int)> job;
                {
                    std::unique_lock<std::mutex> lk(E->jmu);
                    E->jcv.wait(lk, [&] { return E->stop || E->job_gen != seen; });
                    if (E->stop) return;
                    seen = E->job_gen;
                    job = E->job;
                }
                job(i);
                {
                    std::lock_guard<std::mutex> lk(E->jmu);
                    ++E->job_done;
                }
                E->dcv.notify_all();
            }
        });
    }
    return QZGPU_NO_ERROR;
}

void engine_free(Engine* E) {
    {
        std::lock_guard<std::mutex> lk(E->jmu);
        E->stop = true;
    }
    E->jcv.notify_all();
    for (auto& t : E->threads) t.join();
    E->threads.clear();
    for (auto& s : E->lanes) {
        cudaSetDevice(s->device);
        storage_free(s.get());
    }
    E->lanes.clear();
}

int engine_run(Engine* E, bool forward, int nb, const int* n, const unsigned char* const* hin,
               unsigned char* const* hout, const unsigned char* d_in, unsigned char* d_out, int* idx,
               cudaStream_t user_stream) {
    const bool host = hin != nullptr;
    if (!host && user_stream) {
        // inputs produced on the caller's stream must be complete
        cudaError_t e = cudaStreamSynchronize(user_stream);
        if (e != cudaSuccess) return map_cuda_error(e);
    }
    // sub-batches: consecutive whole blocks, at most lane_bytes (a larger block
    // alone); lane 0 takes those above lane_bytes first, the lanes then take
    // the others largest first
    using Sub = SubBatch;
    std::vector<Sub> big, small;
    plan_sub_batches(nb, n, std::min(E->lane_bytes, forward ? E->fwd_sub_bytes : E->inv_sub_bytes), E->lane_bytes,
                     &big, &small);
    std::vector<const Sub*> order;
    for (const Sub& sb : big) order.push_back(&sb);
    for (const Sub& sb : small) order.push_back(&sb);
    long long off = 0;
    for (int b = 0; b < nb; ++b) off += n[b];
    // Output pages of host buffers that nothing has touched yet (fresh
    // allocations) make device-to-host copies fault page by page, several
    // times slower than into resident pages.  A host thread touches one byte
    // per page of every output buffer, sub-batch by sub-batch in the order the
    // lanes take them, while the device works; a lane waits for its
    // sub-batch's pages before it copies the blocks out.  Page-locked outputs
    // are resident already and are not touched.
    const int nsub = (int)order.size();
    std::atomic<int> touched{nsub};  // sub-batches (in `order`) whose pages are touched
    std::mutex tmu;
    std::condition_variable tcv;
    std::thread toucher;
    if (host && off >= kTouchMinBytes && !outputs_pinned(nb, n, hout)) {
        touched = 0;
        toucher = std::thread([&] {
            for (int k = 0; k < nsub; ++k) {
                for (int b = order[k]->b0; b < order[k]->b1; ++b) {
                    // in place (output = input): the caller's pages are
                    // resident and still hold the input
                    volatile unsigned char* p = hout[b];
                    if (hout[b] != hin[b])
                        for (long long o = 0; o < n[b]; o += 4096) p[o] = 0;
                }
                {
                    std::lock_guard<std::mutex> lk(tmu);
                    touched.store(k + 1);
                }
                tcv.notify_all();
            }
        });
    }
    const int K = (int)E->lanes.size();
    std::atomic<int> cursor{0};
    std::atomic<int> first_err{0};
    std::vector<std::vector<long long>> lane_rounds(K);
    std::vector<int> lane_maxr(K, 0), lane_launch(K, 0);
    for (auto& s : E->lanes) {
        s->profile = E->profile;
        s->profile_only = E->profile_only;
    }
    auto run_sub = [&](int lane, const Sub& sb) {
        Storage* S = E->lanes[lane].get();
        const int cnt = sb.b1 - sb.b0;
        int rc;
        if (host) {
            const std::function<void()> wait_out = [&] {
                std::unique_lock<std::mutex> lk(tmu);
                tcv.wait(lk, [&] { return touched.load() > sb.seq; });
            };
            if (forward) {
                rc = encode_host(S, cnt, hin + sb.b0, hout + sb.b0, n + sb.b0, idx + sb.b0, nullptr, nullptr,
                                 &wait_out);
            } else {
                // a lane's inverse sub-batches are queued back to back on its
                // stream (copies in, inverse, copies out) and checked once at
                // the end, so no lane waits for the device between them
                if (!S->inv_chained) inverse_chain_begin(S, S->stream);
                rc = decode_host_chained(S, cnt, hin + sb.b0, hout + sb.b0, n + sb.b0, idx + sb.b0, &wait_out);
            }
        } else {
            rc = forward ? forward_run(S, cnt, n + sb.b0, d_in + sb.off, d_out + sb.off, idx + sb.b0, nullptr,
                                       nullptr, S->stream)
                         : inverse_run(S, cnt, n + sb.b0, idx + sb.b0, d_in + sb.off, d_out + sb.off, S->stream);
        }
        if (rc) {
            int z = 0;
            first_err.compare_exchange_strong(z, rc);
            return;
        }
        lane_launch[lane] += S->stats.kernel_launches;
        if (!forward) return;  // round counts describe forward calls only
        auto& lr = lane_rounds[lane];
        if (lr.size() < S->rounds_active.size()) lr.resize(S->rounds_active.size(), 0);
        for (size_t r = 0; r < S->rounds_active.size(); ++r) lr[r] += S->rounds_active[r];
        lane_maxr[lane] = std::max(lane_maxr[lane], S->stats.rounds);
    };
    {
        std::unique_lock<std::mutex> lk(E->jmu);
        E->job = [&](int lane) {
            cudaSetDevice(E->device);
            if (lane == 0)
                for (const Sub& sb : big)
                    if (!first_err.load()) run_sub(0, sb);
            for (;;) {
                int i = cursor.fetch_add(1);
                if (i >= (int)small.size() || first_err.load()) break;
                run_sub(lane, small[i]);
            }
            Storage* S = E->lanes[lane].get();
            if (S->inv_chained) {
                const int rc = inverse_chain_end(S, S->stream);
                int z = 0;
                if (rc) first_err.compare_exchange_strong(z, rc);
            }
        };
        E->job_done = 0;
        ++E->job_gen;
        E->jcv.notify_all();
        E->dcv.wait(lk, [&] { return E->job_done == K; });
        E->job = nullptr;
    }
    if (toucher.joinable()) toucher.join();
    // merge lane counters (round counts only for a forward call)
    E->stats = qzgpu_stats{};
    if (forward) E->rounds_active.clear();
    long long active = 0;
    for (int i = 0; i < K; ++i) {
        auto& lr = lane_rounds[i];
        if (E->rounds_active.size() < lr.size()) E->rounds_active.resize(lr.size(), 0);
        for (size_t r = 0; r < lr.size(); ++r) {
            E->rounds_active[r] += lr[r];
            active += lr[r];
        }
        E->stats.rounds = std::max(E->stats.rounds, lane_maxr[i]);
        E->stats.kernel_launches += lane_launch[i];
        for (auto& kv : E->lanes[i]->prof) {
            auto& g = E->prof[kv.first];
            g.launches += kv.second.launches;
            g.ms += kv.second.ms;
            g.bytes += kv.second.bytes;
        }
        E->lanes[i]->prof.clear();
    }
    long long N = off;
    E->stats.active_total = active;
    E->stats.alg_bytes = forward ? 15 * N + 28 * active : 12 * N;
    return first_err.load();
}

}  // namespace qz
