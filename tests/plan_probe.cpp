// plan_probe.cpp -- C entry point over the library's batched-launch planner
// (mtgp_gb300/csrc/plan_core.cpp), compiled by tests/test_plan_host.py so
// that planning is checked on the CPU against an independent model.
#include <cstring>
#include <string>

#include "../mtgp_gb300/csrc/plan_core.h"

using namespace mtgp;

extern "C" int probe_plan(const mtgp_work_item_t *items, int nitems, int nstreams,
                          int word_bytes, int can_jump, int64_t chunk_tune, int resident,
                          int64_t *task_cols, int task_cap, int64_t *seg_cols, int seg_cap,
                          int32_t *stage, int stage_cap, int64_t *info, char *err, int errcap) {
    PlanOptions o;
    o.nstreams = nstreams;
    o.word_bytes = (size_t)word_bytes;
    o.can_jump = can_jump != 0;
    o.chunk_tune = chunk_tune;
    o.resident = resident;
    PlanResult r;
    std::string msg;
    const int rc = planCore(items, nitems, o, &r, &msg);
    if (err && errcap > 0) std::snprintf(err, (size_t)errcap, "%s", msg.c_str());
    if (rc) return rc;
    info[0] = (int64_t)r.tasks.size();
    info[1] = (int64_t)r.segs.size();
    info[2] = (int64_t)r.stage_streams.size();
    info[3] = r.chunk;
    info[4] = (int64_t)r.out_bytes;
    info[5] = r.mode;
    if ((int)r.tasks.size() > task_cap || (int)r.segs.size() > seg_cap ||
        (int)r.stage_streams.size() > stage_cap)
        return 1;  // caller retries with room
    for (size_t k = 0; k < r.tasks.size(); k++) {  // 7 columns per task
        const PlanTask &t = r.tasks[k];
        int64_t *c = task_cols + 7 * k;
        c[0] = t.stream; c[1] = t.wb; c[2] = (int64_t)t.run; c[3] = (int64_t)t.off;
        c[4] = (int64_t)t.total; c[5] = t.first; c[6] = t.n;
    }
    for (size_t k = 0; k < r.segs.size(); k++) {  // 3 columns per segment
        int64_t *c = seg_cols + 3 * k;
        c[0] = (int64_t)r.segs[k].out_off; c[1] = (int64_t)r.segs[k].count; c[2] = r.segs[k].kind;
    }
    std::memcpy(stage, r.stage_streams.data(), sizeof(int32_t) * r.stage_streams.size());
    return 0;
}

// The tap-chunk ranges of a jump's parts (partChunk): bounds[0..parts].
extern "C" void probe_part_chunks(int tchunks, int parts, int32_t *bounds) {
    for (int q = 0; q <= parts; q++) bounds[q] = partChunk(q, tchunks, parts);
}
