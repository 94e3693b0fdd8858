// serve_probe.cpp -- drives the serving loop's admission rules and arena
// (mtgp_gb300/csrc/server_core.h) through a simulated trace on the CPU, for
// tests/test_serve_host.py.
#include "../mtgp_gb300/csrc/server_core.h"

using namespace mtgp;

// All requests are pending at the start.  Each round admits one batch into a
// free slot if it can; otherwise it retires an in-flight batch chosen by
// `retire` (cyclically) and frees its streams and arena space.  Outputs per
// request: its batch, arena offset and admission rank; per batch: the round
// it was admitted and retired in.
extern "C" int probe_serve(int nreq, const int32_t *pool, const uint32_t *stream,
                           const uint64_t *skip, const uint64_t *bytes, int nstreams0,
                           int nstreams1, uint64_t budget, int max_batch, int slots,
                           const uint32_t *retire, int nretire, int32_t *batch_of,
                           uint64_t *off_of, int32_t *rank_of, int32_t *batch_admit,
                           int32_t *batch_retire, int *nbatches) {
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
    std::vector<char> busy[2];
    busy[0].assign((size_t)nstreams0, kStreamFree);
    busy[1].assign((size_t)nstreams1, kStreamFree);
    Arena arena;
    arena.init(budget);
    std::vector<std::vector<ServeReq>> inflight;
    std::vector<int> inflight_id;
    int nb = 0, rank = 0, ri = 0, done = 0;
    for (int round = 0; done < nreq; round++) {
        if (round > 100 * nreq + 100) return -1;  // no progress
        std::vector<ServeReq> take;
        if ((int)inflight.size() < slots && !pending.empty())
            admitBatch(pending, busy, arena, max_batch, uint64_t(1) << 17, &take);
        if (!take.empty()) {
            for (const ServeReq &r : take) {
                batch_of[r.ticket] = nb;
                off_of[r.ticket] = r.off;
                rank_of[r.ticket] = rank++;
            }
            batch_admit[nb] = round;
            inflight.push_back(take);
            inflight_id.push_back(nb++);
            continue;
        }
        if (inflight.empty()) return -2;  // stuck with nothing on the GPU
        const size_t j = retire[ri++ % nretire] % inflight.size();
        for (const ServeReq &r : inflight[j]) {
            arena.release(r.off, r.bytes);
            busy[r.pool][r.stream] = kStreamFree;
            done++;
        }
        batch_retire[inflight_id[j]] = round;
        inflight.erase(inflight.begin() + (long)j);
        inflight_id.erase(inflight_id.begin() + (long)j);
    }
    *nbatches = nb;
    return arena.free_bytes() == budget ? 0 : -3;  // everything returned
}
