// plan_core.h -- host-side planning of one batched launch (no CUDA).
//
// Turns work items (mtgp_work_item_t: stream, kind, count, output offset,
// skip) into the tasks of a persistent launch.  Positions count steps from a
// stream's window at launch.
//   - Items of one stream keep the caller's order.
//   - A skip (or an advance-only item) of at least `jump_min` values, when
//     the kernels can jump (`can_jump`), is not generated: the work after it
//     is a new run that starts at that position, reached by jumping the
//     window inside the kernel.  Shorter skips are generated (advance items);
//     generated skips above `max_gen_skip` are rejected.
//   - A run longer than `chunk` is cut into k = ceil(length / chunk)
//     near-equal pieces whose length is rounded up to a multiple of the
//     largest power of two <= chunk / 8 (at most 2^16; the last piece takes
//     the rest); piece c starts at run start + c * piece.
//   - The chunk length is `chunk_tune` when > 0, none when < 0, and
//     otherwise the next power of two >= (all generated values / resident
//     CTAs), at least 2^17.
//   - The tasks of one stream all start from its window and run in
//     parallel.  A stream with one task writes its window back directly; with
//     several, the last one (in stream order) writes to a staging slot that is
//     copied back after the launch, the others write nothing.
//   - Tasks are ordered longest first, a start jump counting as `jump_min`
//     values (about its cost).
// The kernel-side jump of a task is X^run then X^off (either may be 0).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/mtgp_gpu.h"

namespace mtgp {

// First tap chunk of part q of a jump split into `parts` over `tchunks`
// chunks (part q covers [partChunk(q), partChunk(q + 1))).  A part generates
// the sequence up to its last chunk and correlates only its own, so the
// later parts are the longer ones: the rounding gives the extra chunks to
// the earlier parts (11 chunks in 4 parts: 3, 3, 3, 2 rather than 2, 3, 3, 3).
inline int partChunk(int q, int tchunks, int parts) {
    const int rem = tchunks % parts;
    return q * (tchunks / parts) + (q < rem ? q : rem);
}

struct PlanOptions {
    int nstreams = 0;
    size_t word_bytes = 4;          // bytes of one output value
    bool can_jump = false;          // in-kernel jumps available
    uint64_t jump_min = uint64_t(1) << 17;
    uint64_t max_gen_skip = uint64_t(1) << 34;
    int64_t chunk_tune = 0;         // > 0 fixed, < 0 never cut, 0 automatic
    int resident = 1;               // resident CTAs of the jumping kernel
};

// One item of a task: count values of kind (-1 = advance without output).
struct PlanSeg {
    uint64_t out_off;
    uint64_t count;
    int32_t kind;
};

struct PlanTask {
    int32_t stream;
    int32_t wb;           // -1 = back to the stream, -2 = none, k >= 0 = staging slot k
    uint64_t run, off;    // start position = run + off
    uint64_t total;       // values the task steps through
    uint32_t first, n;    // its items: segs[first, first + n)
};

struct PlanResult {
    std::vector<PlanTask> tasks;        // longest first
    std::vector<PlanSeg> segs;
    std::vector<int32_t> stage_streams; // staging slot k -> stream
    int64_t chunk = 0;                  // chunk length used (0 = no run was cut)
    uint64_t out_bytes = 0;             // max over items of offset + size
    int mode = -1;                      // shared kind of all values, -1 all advance, -2 mixed
};

// Returns MTGP_OK or an MTGP_ERR_* code with a message in *err.
int planCore(const mtgp_work_item_t *items, int nitems, const PlanOptions &o, PlanResult *r,
             std::string *err);

}  // namespace mtgp
