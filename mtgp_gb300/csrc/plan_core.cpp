// plan_core.cpp -- see plan_core.h.  Flat arrays throughout: the per-item
// work is a few appends, so serving loops can plan thousands of requests
// per batch cheaply.
#include "plan_core.h"

#include <algorithm>
#include <cstdarg>
#include <cstdio>

namespace mtgp {

namespace {

int fail(std::string *err, int code, const char *fmt, ...) {
    char buf[200];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (err) *err = buf;
    return code;
}

// Piece lengths of cut runs are multiples of a grain: the largest power of
// two <= chunk / 8, at most 2^16 values.
uint64_t pieceGrain(uint64_t chunk) {
    uint64_t g = 1;
    while (g * 2 <= chunk / 8 && g < (uint64_t(1) << 16)) g *= 2;
    return g;
}

// A run: consecutive generated work of one stream starting at `start`.
struct Run {
    int32_t stream;
    uint64_t start, total;
    uint32_t first, n;  // segs of the run in the run-segment array
};

}  // namespace

int planCore(const mtgp_work_item_t *items, int nitems, const PlanOptions &o, PlanResult *r,
             std::string *err) {
    r->tasks.clear();
    r->segs.clear();
    r->stage_streams.clear();
    r->chunk = 0;
    r->out_bytes = 0;
    r->mode = -1;
    if (nitems < 0 || (nitems > 0 && !items))
        return fail(err, MTGP_ERR_INVALID, "bad item list (%d items)", nitems);
    // the items with work, grouped by stream in item order: keys (stream <<
    // 32 | item) sorted, so the cost follows the items, not the streams
    // (buffers are reused across calls of a thread: a server plans every
    // batch)
    thread_local std::vector<uint64_t> keys;
    keys.clear();
    for (int k = 0; k < nitems; k++) {
        const mtgp_work_item_t &it = items[k];
        if (it.stream >= (uint32_t)o.nstreams)
            return fail(err, MTGP_ERR_INVALID, "item %d: stream %u out of range", k,
                        (unsigned)it.stream);
        if (it.kind < -1 || it.kind > 4)
            return fail(err, MTGP_ERR_INVALID, "item %d: unknown kind %d", k, (int)it.kind);
        if (it.kind >= 0) {
            if (it.out_offset % o.word_bytes)
                return fail(err, MTGP_ERR_INVALID, "item %d: offset not a multiple of %llu", k,
                            (unsigned long long)o.word_bytes);
            if (it.count > (~uint64_t(0) - it.out_offset) / o.word_bytes)
                return fail(err, MTGP_ERR_INVALID, "item %d: output range overflows", k);
        }
        if (it.count == 0 && it.skip == 0) continue;
        keys.push_back((uint64_t)it.stream << 32 | (uint32_t)k);
    }
    if (keys.size() * 8 < (size_t)o.nstreams) {
        std::sort(keys.begin(), keys.end());
    } else {  // many items: a counting sort by stream (stable)
        thread_local std::vector<int32_t> head;
        thread_local std::vector<uint64_t> by;
        head.assign((size_t)o.nstreams + 1, 0);
        for (uint64_t key : keys) head[(key >> 32) + 1]++;
        for (int st = 0; st < o.nstreams; st++) head[st + 1] += head[st];
        by.resize(keys.size());
        for (uint64_t key : keys) by[(size_t)head[key >> 32]++] = key;
        keys.swap(by);
    }
    // runs, and the generated segments of each run
    thread_local std::vector<Run> runs;
    thread_local std::vector<PlanSeg> rseg;
    runs.clear();
    rseg.clear();
    rseg.reserve(keys.size() + 8);
    uint64_t grand = 0;
    for (size_t q0 = 0, q1; q0 < keys.size(); q0 = q1) {
        const int s = (int)(keys[q0] >> 32);
        for (q1 = q0; q1 < keys.size() && (int)(keys[q1] >> 32) == s; q1++) {
        }
        Run cur{s, 0, 0, (uint32_t)rseg.size(), 0};
        uint64_t pos = 0;
        for (size_t q = q0; q < q1; q++) {
            const int k = (int)(uint32_t)keys[q];
            const mtgp_work_item_t &it = items[k];
            uint64_t skip = it.skip, count = it.count;
            if (it.kind < 0) {  // advance only: all of it is a skip
                skip += count;
                count = 0;
                if (skip < it.skip) return fail(err, MTGP_ERR_INVALID, "item %d: skip overflows", k);
            }
            if (pos + skip < pos || pos + skip + count < pos + skip)
                return fail(err, MTGP_ERR_INVALID, "item %d: stream position overflows 64 bits", k);
            if (skip >= o.jump_min && o.can_jump) {
                if (cur.n) {
                    grand += cur.total;
                    runs.push_back(cur);
                }
                pos += skip;
                cur = Run{s, pos, 0, (uint32_t)rseg.size(), 0};
            } else if (skip) {
                if (skip > o.max_gen_skip)
                    return fail(err, MTGP_ERR_UNSUPPORTED,
                                "item %d: skip of %llu values would be generated (no in-kernel "
                                "jump for this exponent); jump the stream instead",
                                k, (unsigned long long)skip);
                rseg.push_back(PlanSeg{0, skip, -1});
                cur.n++;
                cur.total += skip;
                pos += skip;
            }
            if (count) {
                rseg.push_back(PlanSeg{it.out_offset, count, it.kind});
                cur.n++;
                cur.total += count;
                pos += count;
                r->out_bytes = std::max(r->out_bytes, it.out_offset + count * o.word_bytes);
            }
        }
        if (cur.n || cur.start) {
            if (!cur.n) {  // ends with a jump: a task that only jumps
                rseg.push_back(PlanSeg{0, 0, -1});
                cur.n = 1;
            }
            grand += cur.total;
            runs.push_back(cur);
        }
    }
    int64_t chunk = 0;
    if (o.can_jump) {
        if (o.chunk_tune > 0) {
            chunk = o.chunk_tune;
        } else if (o.chunk_tune == 0) {
            // a task longer than the average load of one CTA slot would set
            // the length of the whole launch
            const uint64_t per = grand / (uint64_t)std::max(o.resident, 1);
            chunk = (int64_t)std::max<uint64_t>(uint64_t(1) << 17, o.jump_min);
            while ((uint64_t)chunk < per) chunk <<= 1;
        }
    }
    // cut runs into tasks; per stream, mark write-back
    const uint64_t grain = chunk > 0 ? pieceGrain((uint64_t)chunk) : 1;
    r->segs.reserve(rseg.size() + runs.size());
    bool cut = false;
    for (size_t r0 = 0, r1; r0 < runs.size(); r0 = r1) {
        for (r1 = r0; r1 < runs.size() && runs[r1].stream == runs[r0].stream; r1++) {
        }
        const size_t first_task = r->tasks.size();
        for (size_t ri = r0; ri < r1; ri++) {
            const Run &R = runs[ri];
            // a run longer than one chunk becomes k = ceil(total / chunk)
            // near-equal pieces, rounded up to a multiple of the grain so
            // that the pieces' offsets (and jump polynomials) recur across
            // requests; the last piece takes the rest
            uint64_t k = 1, piece = R.total;
            if (chunk > 0 && R.total > (uint64_t)chunk) {
                k = (R.total + (uint64_t)chunk - 1) / (uint64_t)chunk;
                piece = (R.total + k - 1) / k;
                piece = (piece + grain - 1) / grain * grain;
                k = (R.total + piece - 1) / piece;
                if (k > 1) cut = true;
            }
            uint32_t si = R.first;     // segment of R being cut
            const uint32_t se = R.first + R.n;
            uint64_t used = 0;         // values of it already taken
            for (uint64_t c = 0; c < k; c++) {
                PlanTask t{};
                t.stream = R.stream;
                t.run = R.start;
                t.off = c * piece;
                t.first = (uint32_t)r->segs.size();
                uint64_t want = (c + 1 == k) ? ~uint64_t(0) : piece;
                while (si < se && (want || rseg[si].count == used)) {
                    PlanSeg g = rseg[si];
                    const uint64_t take = std::min(g.count - used, want);
                    if (g.kind >= 0) g.out_off += used * o.word_bytes;
                    g.count = take;
                    r->segs.push_back(g);
                    t.total += take;
                    want -= take;
                    used += take;
                    if (used == rseg[si].count) {
                        si++;
                        used = 0;
                    }
                }
                t.n = (uint32_t)r->segs.size() - t.first;
                r->tasks.push_back(t);
            }
        }
        const size_t m = r->tasks.size() - first_task;
        for (size_t q = first_task; q < r->tasks.size(); q++)
            r->tasks[q].wb = m == 1 ? -1
                                    : (q + 1 == r->tasks.size() ? (int32_t)r->stage_streams.size()
                                                                : -2);
        if (m > 1) r->stage_streams.push_back(runs[r0].stream);
    }
    r->chunk = cut ? chunk : 0;
    // longest task first, a jump counted as jump_min generated values (about
    // its cost)
    const uint64_t jw = o.can_jump ? o.jump_min : 0;
    auto cost = [jw](const PlanTask &t) {
        return t.total + jw * ((t.run ? 1u : 0u) + (t.off ? 1u : 0u));
    };
    // by (cost descending, position): a stable order, sorted as plain pairs
    thread_local std::vector<std::pair<uint64_t, uint32_t>> ord;
    thread_local std::vector<PlanTask> sorted;
    ord.resize(r->tasks.size());
    for (size_t q = 0; q < r->tasks.size(); q++)
        ord[q] = {~cost(r->tasks[q]), (uint32_t)q};
    std::sort(ord.begin(), ord.end());
    sorted.resize(r->tasks.size());
    for (size_t q = 0; q < ord.size(); q++) sorted[q] = r->tasks[ord[q].second];
    r->tasks.swap(sorted);
    int mode = -3;
    for (const PlanSeg &g : r->segs)
        if (g.count) mode = (mode == -3 || mode == g.kind) ? g.kind : -2;
    r->mode = mode == -3 ? -1 : mode;
    return MTGP_OK;
}

}  // namespace mtgp
