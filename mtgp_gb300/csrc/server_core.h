// server_core.h -- the serving loop's admission rules and output arena (no
// CUDA), shared by server.cpp and the CPU tests.
#pragma once
#include <algorithm>
#include <chrono>
#include <cstdint>
#include <deque>
#include <iterator>
#include <map>
#include <utility>
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

inline std::vector<std::pair<int, uint32_t>> &waitingScratch() {
    static thread_local std::vector<std::pair<int, uint32_t>> v;
    return v;
}

// Per-stream marks during one admission pass (all kStreamFree between
// passes): not in the batch being formed, in it, in it but closed to more
// requests.
enum : char { kStreamFree = 0, kStreamForming = 1, kStreamClosed = 2 };

// Move the next batch's requests from `pending` to `take`, in one pass:
//   - first come, first served: admission stops at the first request whose
//     output would take the batch past `limit` bytes, or past `soft` bytes
//     when it is not the batch's first request.  The batch's outputs are laid
//     out back to back, each rounded up to the arena's 256-byte granule;
//     r.off is the offset in the batch's block, which is placed in the arena
//     later (Arena::alloc);
//   - a stream may have earlier batches still on the GPU: if `held(r)` says
//     so for its first request in the pass, the stream waits (with all its
//     later requests) for them to finish; otherwise its requests join, and
//     the caller orders the new batch after those batches (StreamOrder);
//   - several requests of one stream may join the batch, in order, except
//     that a skip of at least `jump_skip` only opens a stream's part of a
//     batch (its jump is then X^skip from the window, a polynomial shared by
//     many requests, instead of X^(an arbitrary position)); the stream's
//     later requests then wait for the next batch;
//   - at most `max_batch` requests, and at most `max_scan` pending requests
//     looked at (a bound on the time the caller holds its lock).
// mark[pool][stream] is scratch.  Returns the block's size in bytes.
template <class Held>
uint64_t admitBatch(std::deque<ServeReq> &pending, std::vector<char> *mark, int max_batch,
                    uint64_t jump_skip, uint64_t limit, uint64_t soft, Held held,
                    std::vector<ServeReq> *take, size_t max_scan = ~size_t(0)) {
    take->clear();
    std::vector<std::pair<int, uint32_t>> &waiting = waitingScratch();
    waiting.clear();
    uint64_t used = 0;
    auto w = pending.begin(), it = pending.begin();
    for (size_t scanned = 0;
         it != pending.end() && (int)take->size() < max_batch && scanned < max_scan;
         ++it, ++scanned) {
        char &m = mark[it->pool][it->stream];
        if (m == kStreamFree && held(*it)) {
            m = kStreamClosed;
            waiting.emplace_back(it->pool, it->stream);
        }
        if (m == kStreamForming && it->skip >= jump_skip) m = kStreamClosed;
        if (m == kStreamClosed) {
            if (w != it) *w = *it;
            ++w;
            continue;
        }
        const uint64_t n = Arena::round(it->bytes);
        if (n > limit - used || (!take->empty() && n > soft - std::min(used, soft))) break;
        it->off = used;
        used += n;
        m = kStreamForming;
        take->push_back(*it);
    }
    pending.erase(w, it);
    for (const ServeReq &r : *take) mark[r.pool][r.stream] = kStreamFree;
    for (const auto &ps : waiting) mark[ps.first][ps.second] = kStreamFree;
    return used;
}

// Requests the next batch may take: max_batch; under a backlog (`backlog`)
// a quarter of what waits, at least a quarter of max_batch and at least one,
// so that a burst gets full batches while a steady load near capacity gets
// batches just large enough to keep up (with half of what waits, a load at
// 0.9 of capacity still tipped into full batches in some runs).
inline int batchCap(size_t pending, int max_batch, bool backlog) {
    if (!backlog) return max_batch;
    const size_t part = pending / 4;
    const int want = part > (size_t)max_batch ? max_batch : (int)part;
    return std::min(max_batch, std::max({1, max_batch / 4, want}));
}

// Output bytes the next batch may take: pending_bytes / 8, at least an
// eighth and at most half of the arena.  Under a burst the batches are large
// (fewer chains of batches on the GPU); a steady load keeps batches of an
// eighth of the arena, small enough that it sustains 0.9 of a burst's rate
// at low latency (a fixed half of the arena tipped such a load into large
// batches and 5-7 ms latency; a fixed eighth ran a burst 5 % slower).
inline uint64_t batchBytes(uint64_t pending_bytes, uint64_t arena) {
    return std::min(arena / 2, std::max(arena / 8, pending_bytes / 8));
}

// The order of batches on the GPU: a batch that holds requests of a stream
// must run after that stream's earlier batches, which read and write the
// stream's window.  Each stream remembers its latest batch by a caller-chosen
// tag (non-zero); deps[pool] receives the distinct tags of those earlier
// batches, through the pool's streams, that `live(tag)` still reports in
// flight.
struct StreamOrder {
    std::vector<uint64_t> last[2];
    uint64_t latest(const ServeReq &r) const { return last[r.pool][r.stream]; }
    void init(size_t n0, size_t n1) {
        last[0].assign(n0, 0);
        last[1].assign(n1, 0);
    }
    template <class Live>
    void order(const std::vector<ServeReq> &take, uint64_t tag, Live live,
               std::vector<uint64_t> deps[2]) {
        deps[0].clear();
        deps[1].clear();
        for (const ServeReq &r : take) {
            uint64_t &l = last[r.pool][r.stream];
            std::vector<uint64_t> &d = deps[r.pool];
            if (l && l != tag && live(l) && std::find(d.begin(), d.end(), l) == d.end())
                d.push_back(l);
            l = tag;
        }
    }
};

}  // namespace mtgp
