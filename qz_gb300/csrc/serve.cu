// Serving form: block requests (forward or inverse BWT) from any number of
// host threads are admitted into device-resident scratch slots and batched
// continuously.
//
// qz's callers are concurrent: rayon workers per block, up to four chunk
// threads, three or four decoder threads (crates/qz-lib/src/compression/
// compress_impl.rs:364-387, decompress_impl.rs:666-689).  Instead of one GPU
// call per block, the server keeps K storages (slots) resident on the device,
// sized so that K slots fit the HBM budget; K worker threads each own a slot
// and a stream.  A worker that becomes free takes every waiting request of the
// direction at the head of the queue (in arrival order) that fits its slot,
// runs them as one batch, and completes them.  Requests that arrive while
// batches are on the GPU are admitted as soon as a slot is free, and batches
// of different slots overlap on the device.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "engine.h"

namespace qz {
namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    int op;  // 0 forward, 1 inverse
    const unsigned char* in;
    unsigned char* out;
    int n;
    int index;
    Clock::time_point t_submit, t_start, t_done;
    int status = 0;
    int index_out = 0;
    bool done = false;
};

}  // namespace

struct Server {
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<long long> pending;
    std::unordered_map<long long, std::unique_ptr<Request>> reqs;
    std::vector<std::unique_ptr<Storage>> slots;
    std::vector<std::thread> workers;
    bool stop = false;
    long long next_ticket = 0;
    long long slot_bytes = 0;
    int slot_blocks = 0;
    // counters
    long long batches = 0, completed = 0, max_batch = 0, busy = 0, max_busy = 0;

    void worker(int i);
};

void Server::worker(int i) {
    Storage* S = slots[i].get();
    cudaSetDevice(S->device);  // a new thread starts on device 0
    std::vector<long long> take;
    std::vector<const unsigned char*> ins;
    std::vector<unsigned char*> outs;
    std::vector<int> ns, idx;
    for (;;) {
        take.clear();
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_work.wait(lk, [&] { return stop || !pending.empty(); });
            if (pending.empty()) return;  // stop requested and nothing left
            int op = reqs[pending.front()]->op;
            long long bytes = 0;
            for (auto it = pending.begin(); it != pending.end() && (int)take.size() < slot_blocks;) {
                Request* r = reqs[*it].get();
                if (r->op == op && bytes + r->n <= slot_bytes) {
                    bytes += r->n;
                    take.push_back(*it);
                    it = pending.erase(it);
                } else {
                    ++it;
                }
            }
            ++batches;
            max_batch = std::max<long long>(max_batch, (long long)take.size());
            ++busy;
            max_busy = std::max(max_busy, busy);
            ins.clear();
            outs.clear();
            ns.clear();
            idx.clear();
            auto now = Clock::now();
            for (long long t : take) {
                Request* r = reqs[t].get();
                r->t_start = now;
                ins.push_back(r->in);
                outs.push_back(r->out);
                ns.push_back(r->n);
                idx.push_back(r->index);
            }
        }
        int nb = (int)take.size();
        int op = 0;
        {
            std::lock_guard<std::mutex> lk(mu);
            op = reqs[take[0]]->op;
        }
        int rc;
        {
            std::lock_guard<std::mutex> lk(S->mu);
            rc = op == 0 ? encode_host(S, nb, ins.data(), outs.data(), ns.data(), idx.data(), nullptr, nullptr)
                         : decode_host(S, nb, ins.data(), outs.data(), ns.data(), idx.data());
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            auto now = Clock::now();
            for (int b = 0; b < nb; ++b) {
                Request* r = reqs[take[b]].get();
                r->status = rc;
                r->index_out = op == 0 ? idx[b] : r->index;
                r->t_done = now;
                r->done = true;
            }
            completed += nb;
            --busy;
        }
        cv_done.notify_all();
    }
}

}  // namespace qz

struct qzgpu_server : public qz::Server {};

extern "C" {

int qzgpu_server_create(qzgpu_server** out, long long hbm_budget_bytes, int max_slots, long long slot_bytes,
                        int slot_blocks) {
    using namespace qz;
    if (!out) return QZGPU_BAD_PARAMETER;
    *out = nullptr;
    if (slot_bytes <= 0) slot_bytes = 64ll << 20;
    if (slot_blocks <= 0) slot_blocks = 256;
    if (max_slots <= 0) max_slots = 4;
    if (slot_bytes > QZGPU_MAX_BATCH_BYTES) return QZGPU_BAD_PARAMETER;
    int rc = qzgpu_init(0);
    if (rc) return rc;
    size_t free_b = 0, total_b = 0;
    cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess) return map_cuda_error(e);
    long long budget = hbm_budget_bytes > 0 ? std::min<long long>(hbm_budget_bytes, (long long)free_b)
                                            : (long long)(free_b * 0.8);
    long long per = (long long)storage_device_bytes(slot_bytes, slot_blocks);
    int k = (int)std::min<long long>(max_slots, budget / std::max(per, 1ll));
    if (k < 1) return QZGPU_GPU_NOT_ENOUGH_MEMORY;
    auto* srv = new (std::nothrow) qzgpu_server();
    if (!srv) return QZGPU_NOT_ENOUGH_MEMORY;
    srv->slot_bytes = slot_bytes;
    srv->slot_blocks = slot_blocks;
    for (int i = 0; i < k; ++i) {
        auto s = std::make_unique<Storage>();
        rc = storage_init(s.get(), slot_bytes, slot_blocks);
        if (rc) {
            for (auto& x : srv->slots) storage_free(x.get());
            delete srv;
            return rc;
        }
        srv->slots.push_back(std::move(s));
    }
    for (int i = 0; i < k; ++i) srv->workers.emplace_back([srv, i] { srv->worker(i); });
    *out = srv;
    return QZGPU_NO_ERROR;
}

int qzgpu_server_slots(const qzgpu_server* srv) { return srv ? (int)srv->slots.size() : QZGPU_BAD_PARAMETER; }

long long qzgpu_server_submit(qzgpu_server* srv, int op, const unsigned char* in, unsigned char* out, int n,
                              int index) {
    using namespace qz;
    if (!srv || (op != 0 && op != 1) || n < 0 || (n > 0 && (!in || !out))) return QZGPU_BAD_PARAMETER;
    if (n > srv->slot_bytes) return QZGPU_BAD_PARAMETER;
    if (op == 1 && n > 0 && (index < 1 || index > n)) return QZGPU_DATA_CORRUPT;
    auto r = std::make_unique<Request>();
    r->op = op;
    r->in = in;
    r->out = out;
    r->n = n;
    r->index = index;
    r->t_submit = Clock::now();
    long long t;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        if (srv->stop) return QZGPU_BAD_PARAMETER;
        t = srv->next_ticket++;
        if (n <= 1) {
            // nothing to sort: done at once (bsc.rs:162-164 returns early for empty input)
            if (n == 1) out[0] = in[0];
            r->index_out = n;
            r->t_start = r->t_done = r->t_submit;
            r->done = true;
            srv->reqs[t] = std::move(r);
            srv->completed++;
        } else {
            srv->reqs[t] = std::move(r);
            srv->pending.push_back(t);
        }
    }
    srv->cv_work.notify_one();
    srv->cv_done.notify_all();
    return t;
}

int qzgpu_server_wait(qzgpu_server* srv, long long ticket, int timeout_ms, int* status, int* index_out,
                      double* latency_ms, double* queue_ms) {
    using namespace qz;
    if (!srv) return QZGPU_BAD_PARAMETER;
    std::unique_lock<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(ticket);
    if (it == srv->reqs.end()) return QZGPU_BAD_PARAMETER;
    Request* r = it->second.get();
    auto pred = [&] { return r->done; };
    if (timeout_ms < 0) {
        srv->cv_done.wait(lk, pred);
    } else if (!srv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred)) {
        return 0;
    }
    if (status) *status = r->status;
    if (index_out) *index_out = r->index_out;
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    if (queue_ms) *queue_ms = std::chrono::duration<double, std::milli>(r->t_start - r->t_submit).count();
    srv->reqs.erase(it);
    return 1;
}

int qzgpu_server_stats(const qzgpu_server* srv, long long* out, int max) {
    if (!srv || max < 0 || (max > 0 && !out)) return QZGPU_BAD_PARAMETER;
    auto* s = const_cast<qzgpu_server*>(srv);
    std::lock_guard<std::mutex> lk(s->mu);
    long long v[6] = {s->completed, s->batches, s->max_batch, s->max_busy, (long long)s->pending.size(),
                      (long long)s->slots.size()};
    for (int i = 0; i < max && i < 6; ++i) out[i] = v[i];
    return 6;
}

int qzgpu_server_destroy(qzgpu_server* srv) {
    using namespace qz;
    if (!srv) return QZGPU_BAD_PARAMETER;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->stop = true;
    }
    srv->cv_work.notify_all();
    for (auto& t : srv->workers) t.join();
    for (auto& s : srv->slots) {
        cudaSetDevice(s->device);
        storage_free(s.get());
    }
    delete srv;
    return QZGPU_NO_ERROR;
}

}  // extern "C"
