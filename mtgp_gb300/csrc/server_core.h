// server_core.h -- the serving loop's admission rules and output arena (no
// CUDA), shared by server.cpp and the CPU tests.
#pragma once
#include <chrono>
#include <cstdint>
#include <deque>
#include <iterator>
#include <map>
#include <vector>

namespace mtgp {

// First-fit allocator over the output arena, 256-byte granules.
class Arena {
  public:
    void init(uint64_t n) {
        size_ = n;
        free_.clear();
        free_[0] = n;
    }
    static uint64_t round(uint64_t n) { return (n + 255) & ~uint64_t(255); }
    bool alloc(uint64_t n, uint64_t *off) {
        n = round(n);
        if (n == 0) {
            *off = 0;
            return true;
        }
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            *off = it->first;
            const uint64_t rest = it->second - n, at = it->first + n;
            free_.erase(it);
            if (rest) free_[at] = rest;
            return true;
        }
        return false;
    }
    void release(uint64_t off, uint64_t n) {
        n = round(n);
        if (n == 0) return;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    uint64_t size() const { return size_; }
    uint64_t free_bytes() const {
        uint64_t f = 0;
        for (const auto &kv : free_) f += kv.second;
        return f;
    }

  private:
    uint64_t size_ = 0;
    std::map<uint64_t, uint64_t> free_;  // offset -> length of each free block
};

struct ServeReq {
    uint64_t ticket;
    int pool;
    uint32_t stream;
    int kind;
    uint64_t skip, count, bytes, off;
    void *dst;
    bool keep;  // no destination: the result stays in the arena until released
    std::chrono::steady_clock::time_point t_submit;
};

// Stream states during admission: free, in a batch on the GPU, in the batch
// being formed, in the batch being formed but closed to more requests.
enum : char { kStreamFree = 0, kStreamBusy = 1, kStreamForming = 2, kStreamClosed = 3 };

// Move the next batch's requests from `pending` to `take`, in one pass:
//   - first come, first served: admission stops at the first request whose
//     output does not fit in the arena;
//   - a request whose stream has work on the GPU waits (it stays pending, in
//     order, with every later request of that stream);
//   - several requests of one stream may join the batch, in order, except
//     that a skip of at least `jump_skip` only opens a stream's part of a
//     batch (its jump is then X^skip from the window, a polynomial shared by
//     many requests, instead of X^(an arbitrary position));
//   - at most `max_batch` requests, and at most `max_scan` pending requests
//     looked at (a bound on the time the caller holds its lock when the
//     backlog is long and mostly waits for streams on the GPU).
// busy[pool][stream] holds the stream states; admitted streams end as busy.
inline void admitBatch(std::deque<ServeReq> &pending, std::vector<char> *busy, Arena &arena,
                       int max_batch, uint64_t jump_skip, std::vector<ServeReq> *take,
                       size_t max_scan = ~size_t(0)) {
    take->clear();
    auto w = pending.begin(), it = pending.begin();
    for (size_t scanned = 0;
         it != pending.end() && (int)take->size() < max_batch && scanned < max_scan;
         ++it, ++scanned) {
        char &b = busy[it->pool][it->stream];
        if (b == kStreamForming && it->skip >= jump_skip) b = kStreamClosed;
        if (b == kStreamBusy || b == kStreamClosed) {
            if (w != it) *w = *it;
            ++w;
            continue;
        }
        uint64_t off = 0;
        if (!arena.alloc(it->bytes, &off)) break;
        it->off = off;
        b = kStreamForming;
        take->push_back(*it);
    }
    pending.erase(w, it);
    // (a stream is only closed after it joined, so this reaches all of them)
    for (const ServeReq &r : *take) busy[r.pool][r.stream] = kStreamBusy;
}

}  // namespace mtgp
