// Serving form: block requests (forward or inverse BWT) from any number of
// host threads are admitted into device-resident scratch slots and batched
// continuously.
//
// qz's callers are concurrent: rayon workers per block, up to four chunk
// threads, three or four decoder threads (crates/qz-lib/src/compression/
// compress_impl.rs:364-387, decompress_impl.rs:666-689).  Instead of one GPU
// call per block, the server keeps storages (slots) resident on the device,
// each with a worker thread and a stream.  A worker that becomes free takes
// every waiting request of the direction at the head of the queue (in arrival
// order) that fits its slot, runs them as one batch, and completes them;
// requests that arrive while batches are on the GPU are admitted as soon as a
// slot is free, and batches of different slots overlap on the device.
//
// Admission by free HBM: the server starts with one slot.  While requests wait
// and every slot is busy, an admission thread adds a slot if the slots' device
// bytes stay within the server's budget AND the free HBM it reads at that
// moment (cudaMemGetInfo) covers one more slot plus a reserve left to other
// users of the GPU.  Otherwise the requests wait for a busy slot; the
// admission thread reads free HBM again after a short pause.
//
// Results are per request: a batch whose inverse fails for one block (an
// index or BWT that cannot be inverted, bsc.rs:411-433 turns it into an error
// for that call) fails that request alone; its batch-mates complete normally.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "engine.h"
#include "tickets.h"

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
    bool claimed = false;  // a thread waits for it (TicketBook)
};

constexpr long long kReserveBytes = 256ll << 20;        // free HBM an admission leaves to others
constexpr auto kAdmitRetry = std::chrono::milliseconds(2);  // pause before free HBM is read again

}  // namespace

struct Server {
    std::mutex mu;
    std::condition_variable cv_work, cv_done, cv_admit;
    std::deque<Request*> pending;  // in arrival order; owned by the ticket book
    TicketBook<Request> book;
    std::vector<std::unique_ptr<Storage>> slots;  // reserved to max_slots: never reallocated
    std::vector<std::thread> workers;
    std::thread admitter;
    bool stop = false;
    long long slot_bytes = 0;
    int slot_blocks = 0;
    int max_slots = 0;
    long long budget = 0;    // device bytes all slots may hold together
    long long per_slot = 0;  // device bytes of one slot (qzgpu_storage_bytes of its capacity)
    int idle = 0;            // workers waiting for work
    // counters
    long long batches = 0, completed = 0, max_batch = 0, busy = 0, max_busy = 0, refused = 0;

    void worker(Storage* S);
    void admit_loop();
    bool want_slot() const {
        return !stop && !pending.empty() && idle == 0 && (int)slots.size() < max_slots &&
               (long long)(slots.size() + 1) * per_slot <= budget;
    }
    void add_slot(std::unique_ptr<Storage> s) {  // caller holds mu
        Storage* S = s.get();
        slots.push_back(std::move(s));
        workers.emplace_back([this, S] { worker(S); });
    }
};

void Server::admit_loop() {
    std::unique_lock<std::mutex> lk(mu);
    int dev = slots.empty() ? 0 : slots[0]->device;
    cudaSetDevice(dev);  // a new thread starts on device 0
    for (;;) {
        cv_admit.wait(lk, [&] { return stop || want_slot(); });
        if (stop) return;
        lk.unlock();
        size_t free_b = 0, total_b = 0;
        bool ok = cudaMemGetInfo(&free_b, &total_b) == cudaSuccess &&
                  (long long)free_b >= per_slot + kReserveBytes;
        std::unique_ptr<Storage> s;
        if (ok) {
            s = std::make_unique<Storage>();
            if (storage_init(s.get(), slot_bytes, slot_blocks) != QZGPU_NO_ERROR) {
                ok = false;
                s.reset();
            }
        }
        lk.lock();
        if (ok && !stop) {
            add_slot(std::move(s));
        } else {
            if (s) storage_free(s.get());
            ++refused;
            // not enough free HBM now: the waiting requests go to busy slots
            // as they free up; free HBM is read again after a pause
            cv_admit.wait_for(lk, kAdmitRetry, [&] { return stop; });
        }
    }
}

void Server::worker(Storage* S) {
    cudaSetDevice(S->device);  // a new thread starts on device 0
    std::vector<Request*> take;
    std::vector<const unsigned char*> ins;
    std::vector<unsigned char*> outs;
    std::vector<int> ns, idx, rcs;
    for (;;) {
        take.clear();
        int op = 0;
        {
            std::unique_lock<std::mutex> lk(mu);
            ++idle;
            cv_work.wait(lk, [&] { return stop || !pending.empty(); });
            --idle;
            if (pending.empty()) return;  // stop requested and nothing left
            op = pending.front()->op;
            long long bytes = 0;
            for (auto it = pending.begin(); it != pending.end() && (int)take.size() < slot_blocks;) {
                Request* r = *it;
                if (r->op == op && bytes + r->n <= slot_bytes) {
                    bytes += r->n;
                    take.push_back(r);
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
            for (Request* r : take) {
                r->t_start = now;
                ins.push_back(r->in);
                outs.push_back(r->out);
                ns.push_back(r->n);
                idx.push_back(r->index);
            }
            // requests left behind while every slot works: ask for another slot
            if (want_slot()) cv_admit.notify_one();
        }
        const int nb = (int)take.size();
        rcs.assign(nb, 0);
        int rc;
        {
            std::lock_guard<std::mutex> lk(S->mu);
            rc = op == 0 ? encode_host(S, nb, ins.data(), outs.data(), ns.data(), idx.data(), nullptr, nullptr)
                         : decode_host(S, nb, ins.data(), outs.data(), ns.data(), idx.data(), nullptr, rcs.data());
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            auto now = Clock::now();
            for (int b = 0; b < nb; ++b) {
                Request* r = take[b];
                // an inverse failure names its blocks; any other failure is the batch's
                r->status = (op == 1 && rc == QZGPU_DATA_CORRUPT) ? rcs[b] : rc;
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
    if (slot_bytes > QZGPU_MAX_BATCH_BYTES || max_slots > 64) return QZGPU_BAD_PARAMETER;
    int rc = qzgpu_init(0);
    if (rc) return rc;
    size_t free_b = 0, total_b = 0;
    cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess) return map_cuda_error(e);
    long long budget = hbm_budget_bytes > 0 ? std::min<long long>(hbm_budget_bytes, (long long)free_b)
                                            : (long long)(free_b * 0.8);
    long long per = (long long)storage_device_bytes(slot_bytes, slot_blocks);
    if (per > budget) return QZGPU_GPU_NOT_ENOUGH_MEMORY;
    auto* srv = new (std::nothrow) qzgpu_server();
    if (!srv) return QZGPU_NOT_ENOUGH_MEMORY;
    srv->slot_bytes = slot_bytes;
    srv->slot_blocks = slot_blocks;
    srv->max_slots = max_slots;
    srv->budget = budget;
    srv->per_slot = per;
    srv->slots.reserve(max_slots);
    srv->workers.reserve(max_slots);
    auto s = std::make_unique<Storage>();
    rc = storage_init(s.get(), slot_bytes, slot_blocks);
    if (rc) {
        delete srv;
        return rc;
    }
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->add_slot(std::move(s));
    }
    srv->admitter = std::thread([srv] { srv->admit_loop(); });
    *out = srv;
    return QZGPU_NO_ERROR;
}

int qzgpu_server_slots(const qzgpu_server* srv) {
    if (!srv) return QZGPU_BAD_PARAMETER;
    auto* s = const_cast<qzgpu_server*>(srv);
    std::lock_guard<std::mutex> lk(s->mu);
    return (int)s->slots.size();
}

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
    bool queued = false;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        if (srv->stop) return QZGPU_BAD_PARAMETER;
        Request* rp = r.get();
        if (n <= 1) {
            // nothing to sort: done at once (bsc.rs:162-164 returns early for empty input)
            if (n == 1) out[0] = in[0];
            r->index_out = n;
            r->t_start = r->t_done = r->t_submit;
            r->done = true;
            t = srv->book.add(std::move(r));
            srv->completed++;
        } else {
            t = srv->book.add(std::move(r));
            srv->pending.push_back(rp);
            queued = true;
            if (srv->want_slot()) srv->cv_admit.notify_one();
        }
    }
    if (queued) srv->cv_work.notify_one();
    srv->cv_done.notify_all();
    return t;
}

int qzgpu_server_wait(qzgpu_server* srv, long long ticket, int timeout_ms, int* status, int* index_out,
                      double* latency_ms, double* queue_ms) {
    using namespace qz;
    if (!srv) return QZGPU_BAD_PARAMETER;
    std::unique_lock<std::mutex> lk(srv->mu);
    Request* r = nullptr;
    const int got = srv->book.wait(lk, srv->cv_done, ticket, timeout_ms, &r);
    if (got < 0) return QZGPU_BAD_PARAMETER;  // unknown, released, or another thread waits for it
    if (got == 0) return 0;
    if (status) *status = r->status;
    if (index_out) *index_out = r->index_out;
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    if (queue_ms) *queue_ms = std::chrono::duration<double, std::milli>(r->t_start - r->t_submit).count();
    srv->book.release(ticket);
    return 1;
}

int qzgpu_server_stats(const qzgpu_server* srv, long long* out, int max) {
    if (!srv || max < 0 || (max > 0 && !out)) return QZGPU_BAD_PARAMETER;
    auto* s = const_cast<qzgpu_server*>(srv);
    std::lock_guard<std::mutex> lk(s->mu);
    long long v[7] = {s->completed, s->batches, s->max_batch, s->max_busy, (long long)s->pending.size(),
                      (long long)s->slots.size(), s->refused};
    for (int i = 0; i < max && i < 7; ++i) out[i] = v[i];
    return 7;
}

int qzgpu_server_destroy(qzgpu_server* srv) {
    using namespace qz;
    if (!srv) return QZGPU_BAD_PARAMETER;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->stop = true;
    }
    srv->cv_admit.notify_all();
    srv->cv_work.notify_all();
    if (srv->admitter.joinable()) srv->admitter.join();
    // no slot is added after the admission thread has ended
    for (auto& t : srv->workers) t.join();
    for (auto& s : srv->slots) {
        cudaSetDevice(s->device);
        storage_free(s.get());
    }
    delete srv;
    return QZGPU_NO_ERROR;
}

}  // extern "C"
