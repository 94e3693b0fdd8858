// serve_probe.cpp -- drives the serving loop's admission rules, stream order
// and arena (mtgp_gb300/csrc/server_core.h) through a simulated trace on the
// CPU, for tests/test_serve_host.py.
#include <algorithm>

#include "../mtgp_gb300/csrc/server_core.h"

using namespace mtgp;

// All requests are pending at the start.  Each round does the first of:
//   - admit one batch (at most max_batch requests and budget / 8 bytes,
//     unless one request; all admitted batches not yet placed at most the
//     budget) if fewer than `slots` batches are admitted and not retired;
//     a stream with a batch not yet retired joins only while at least
//     `pipe_backlog` requests are pending;
//   - place the oldest admitted batch not yet placed in the arena, if its
//     block fits;
//   - retire one placed batch whose earlier batches of the same streams are
//     all retired (the GPU runs a batch after them), chosen by `retire`
//     (cyclically), returning its block.
// Outputs per request: its batch, arena offset and admission rank; per
// batch: the rounds it was admitted, placed and retired in, and the batches
// it was ordered after (`slots` entries, -1 padded).
extern "C" int probe_serve(int nreq, const int32_t *pool, const uint32_t *stream,
                           const uint64_t *skip, const uint64_t *bytes, int nstreams0,
                           int nstreams1, uint64_t budget, int max_batch, int slots,
                           int pipe_backlog,
                           const uint32_t *retire, int nretire, int32_t *batch_of,
                           uint64_t *off_of, int32_t *rank_of, int32_t *batch_admit,
                           int32_t *batch_place, int32_t *batch_retire, int32_t *batch_deps,
                           int *nbatches) {
    std::deque<ServeReq> pending;
    for (int k = 0; k < nreq; k++) {
        ServeReq r{};
        r.ticket = (uint64_t)k;
        r.pool = pool[k];
        r.stream = stream[k];
        r.skip = skip[k];
        r.bytes = bytes[k];
        pending.push_back(r);
    }
    std::vector<char> mark[2];
    mark[0].assign((size_t)nstreams0, kStreamFree);
    mark[1].assign((size_t)nstreams1, kStreamFree);
    StreamOrder order;
    order.init((size_t)nstreams0, (size_t)nstreams1);
    Arena arena;
    arena.init(budget);
    struct Batch {
        std::vector<ServeReq> reqs;
        uint64_t bytes = 0, block = 0;
        std::vector<uint64_t> deps[2];  // per pool, tags = batch index + 1
        bool placed = false, retired = false;
    };
    std::vector<Batch> all;
    size_t next_place = 0;
    uint64_t ahead = 0;  // bytes of the admitted batches not yet placed
    int live = 0, rank = 0, ri = 0, done = 0;
    for (int round = 0; done < nreq; round++) {
        if (round > 100 * nreq + 100) return -1;  // no progress
        if (live < slots && !pending.empty()) {
            Batch b;
            const bool pipe = (int)pending.size() >= pipe_backlog;
            b.bytes = admitBatch(
                pending, mark, max_batch, uint64_t(1) << 17, budget - ahead, budget / 8,
                [&](const ServeReq &r) {
                    const uint64_t l = order.latest(r);
                    return !pipe && l && !all[l - 1].retired;
                },
                &b.reqs);
            if (!b.reqs.empty()) {
                const int id = (int)all.size();
                order.order(b.reqs, (uint64_t)id + 1,
                            [&all](uint64_t tag) { return !all[tag - 1].retired; }, b.deps);
                for (uint64_t t : b.deps[1])  // one list of the batches it follows
                    if (std::find(b.deps[0].begin(), b.deps[0].end(), t) == b.deps[0].end())
                        b.deps[0].push_back(t);
                if ((int)b.deps[0].size() > slots) return -4;
                for (const ServeReq &r : b.reqs) {
                    batch_of[r.ticket] = id;
                    rank_of[r.ticket] = rank++;
                }
                for (int k = 0; k < slots; k++)
                    batch_deps[(size_t)id * slots + k] =
                        k < (int)b.deps[0].size() ? (int32_t)(b.deps[0][k] - 1) : -1;
                batch_admit[id] = round;
                ahead += b.bytes;
                all.push_back(std::move(b));
                live++;
                continue;
            }
        }
        if (next_place < all.size()) {
            Batch &b = all[next_place];
            if (arena.alloc(b.bytes, &b.block)) {
                b.placed = true;
                ahead -= b.bytes;
                for (const ServeReq &r : b.reqs) off_of[r.ticket] = b.block + r.off;
                batch_place[next_place++] = round;
                continue;
            }
        }
        std::vector<int> ready;
        for (size_t k = 0; k < all.size(); k++) {
            const Batch &b = all[k];
            if (!b.placed || b.retired) continue;
            bool ok = true;
            for (uint64_t t : b.deps[0]) ok = ok && all[t - 1].retired;
            if (ok) ready.push_back((int)k);
        }
        if (ready.empty()) return -2;  // stuck with nothing that can finish
        const int j = ready[retire[ri++ % nretire] % ready.size()];
        Batch &b = all[(size_t)j];
        arena.release(b.block, b.bytes);
        b.retired = true;
        done += (int)b.reqs.size();
        live--;
        batch_retire[j] = round;
    }
    *nbatches = (int)all.size();
    return arena.free_bytes() == budget ? 0 : -3;  // everything returned
}

// The next batch's request cap (batchCap).
extern "C" int probe_batch_cap(uint64_t pending, int max_batch, int backlog) {
    return batchCap((size_t)pending, max_batch, backlog != 0);
}

// The next batch's byte cap (batchBytes).
extern "C" uint64_t probe_batch_bytes(uint64_t pending_bytes, uint64_t arena) {
    return batchBytes(pending_bytes, arena);
}
