// Ticket book of the serving queue (plain C++, no device code): the requests
// a server holds, by ticket, each collected by exactly one waiting thread.
#pragma once
#include <chrono>
#include <condition_variable>
#include <memory>
#include <mutex>
#include <unordered_map>

namespace qz {

// Req needs two fields: bool done (set by whoever completes it, under the
// owner's mutex, followed by a notify of the owner's condition variable) and
// bool claimed (owned by the book).  Every call is made with the owner's
// mutex held.
template <typename Req>
class TicketBook {
  public:
    long long add(std::unique_ptr<Req> r) {
        const long long t = next_++;
        map_[t] = std::move(r);
        return t;
    }

    Req* find(long long t) {
        auto it = map_.find(t);
        return it == map_.end() ? nullptr : it->second.get();
    }

    size_t size() const { return map_.size(); }

    // Waits (up to timeout_ms; < 0: without limit) until ticket t is done.
    // Returns 1 with *out = the request (read it before release(t)), 0 on
    // timeout (the ticket may be waited for again), or -1 for a ticket that is
    // unknown, already released, or waited for by another thread.  Other
    // threads add tickets while this one waits, so no map iterator is kept
    // across the wait: the request is held by pointer (it does not move when
    // the map rehashes) and released by key.
    int wait(std::unique_lock<std::mutex>& lk, std::condition_variable& cv, long long t, int timeout_ms, Req** out) {
        Req* r = find(t);
        if (!r || r->claimed) return -1;
        r->claimed = true;
        auto pred = [r] { return r->done; };
        if (timeout_ms < 0) {
            cv.wait(lk, pred);
        } else if (!cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred)) {
            r->claimed = false;
            return 0;
        }
        *out = r;
        return 1;
    }

    void release(long long t) { map_.erase(t); }

  private:
    std::unordered_map<long long, std::unique_ptr<Req>> map_;
    long long next_ = 0;
};

}  // namespace qz
