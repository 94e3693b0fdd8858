"""Batched path: many streams, uneven lengths, mixed kinds, one persistent
launch; bit-exact vs the oracle, and each result equals the same request
run alone."""
import numpy as np
import pytest
import torch

from mtgp_gb300.params import jump_table, load_table
from gpu_util import as_np_bits, np_bits

pytestmark = pytest.mark.gpu


def _items(rng, nstreams, nitems, bits, max_count=5000):
    from mtgp_gb300.api import work_items
    streams = rng.integers(0, nstreams, nitems)
    kinds = rng.integers(-1, 5, nitems)
    counts = rng.integers(0, max_count, nitems)
    counts[rng.random(nitems) < 0.1] = rng.integers(1, 300, 1)[0]
    esz = bits // 8
    offs = np.zeros(nitems, dtype=np.int64)
    pos = 0
    for k in range(nitems):
        offs[k] = pos
        if kinds[k] >= 0:
            pos += int(counts[k]) * esz
    return work_items(streams, kinds, counts, offs), streams, kinds, counts, offs, pos


@pytest.mark.parametrize("bits,table", [(32, "mtgp32_fast_11213"), (64, "mtgp64dc_fast_11213")])
@pytest.mark.parametrize("graph", [False, True])
def test_batch_vs_oracle(gpu, orc, bits, table, graph):
    from mtgp_gb300.api import Pool
    from mtgp_gb300.params import params_array, MTGP32Params, MTGP64Params
    rng = np.random.default_rng(7 + bits + graph)
    tbl = load_table(table)
    nstreams = 40
    plist = [tbl[i % 5] for i in range(5)]
    pidx = np.arange(nstreams) % 5
    seeds = np.arange(nstreams) + 100
    pool = Pool.create(plist, seeds, pidx)
    items, streams, kinds, counts, offs, nbytes = _items(rng, nstreams, 120, bits)
    out = torch.zeros(nbytes // 4 + 64, dtype=torch.int32, device="cuda")
    plan = pool.plan(items)
    assert plan.output_bytes <= nbytes
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        if graph:
            plan.graph_launch(out, s)
        else:
            plan.launch(out, s)
    s.synchronize()
    got = out.cpu().numpy().view(np.uint8)
    # oracle: replay items stream by stream in order
    P = MTGP32Params if bits == 32 else MTGP64Params
    parr = params_array(P, plist)
    win = orc.seed_windows(bits, parr, seeds, pidx)
    gens = {}
    for k in range(len(streams)):
        sidx = int(streams[k])
        if sidx not in gens:
            o = orc.gen(plist[pidx[sidx]], seed=int(seeds[sidx]))
            gens[sidx] = o
        o = gens[sidx]
        if kinds[k] < 0:
            o.skip(int(counts[k]))
            continue
        ref = np_bits(o.fill(int(kinds[k]), int(counts[k])), bits).view(np.uint8)
        assert np.array_equal(got[offs[k]:offs[k] + ref.size], ref), k
    w = pool.windows()
    for sidx, o in gens.items():
        assert np.array_equal(w[sidx], o.window()), sidx


def test_batch_equals_alone(gpu, orc):
    """A request's output is the same alone and in the mix."""
    from mtgp_gb300.api import Pool, work_items
    p = load_table("mtgp32_fast_11213")[0]
    tbl = jump_table(32)
    mix = Pool.substreams(p, 1234, 64, tbl)
    alone = Pool.substreams(p, 1234, 64, tbl)
    rng = np.random.default_rng(3)
    counts = rng.integers(1, 20000, 64)
    offs = np.concatenate([[0], np.cumsum(counts)[:-1]]) * 4
    out = torch.zeros(int(counts.sum()), dtype=torch.int32, device="cuda")
    mix.submit(work_items(np.arange(64), np.zeros(64), counts, offs), out)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    for j in (0, 5, 63):
        one = torch.zeros(int(counts[j]), dtype=torch.int32, device="cuda")
        alone.fill_stream(j, 0, one, int(counts[j]))
        torch.cuda.synchronize()
        o = int(offs[j]) // 4
        assert np.array_equal(got[o:o + int(counts[j])], one.cpu().numpy()), j


def test_batch_graph_replay_continues(gpu, orc):
    """Replaying a captured plan continues every stream (state advances)."""
    from mtgp_gb300.api import Pool, work_items
    p = load_table("mtgp32_fast_11213")[0]
    pool = Pool.create([p], np.arange(8) + 1, np.zeros(8))
    counts = np.array([100, 5000, 1, 0, 777, 256, 257, 4096])
    offs = np.concatenate([[0], np.cumsum(counts)[:-1]]) * 4
    plan = pool.plan(work_items(np.arange(8), np.zeros(8), counts, offs))
    out = torch.zeros(int(counts.sum()), dtype=torch.int32, device="cuda")
    s = torch.cuda.Stream()
    gens = [orc.gen(p, seed=i + 1) for i in range(8)]
    for rep in range(3):
        plan.graph_launch(out, s)
        s.synchronize()
        got = out.cpu().numpy().view(np.uint32)
        for i in range(8):
            o = int(offs[i]) // 4
            assert np.array_equal(got[o:o + int(counts[i])], gens[i].fill(0, int(counts[i]))), (rep, i)


def test_batch_rejects_bad_items(gpu):
    from mtgp_gb300._lib import MTGPError
    from mtgp_gb300.api import Pool, work_items
    p = load_table("mtgp32_fast_11213")[0]
    pool = Pool.create([p], [1, 2], [0, 0])
    with pytest.raises(MTGPError):
        pool.plan(work_items([5], [0], [10], [0]))
    with pytest.raises(MTGPError):
        pool.plan(work_items([0], [0], [10], [2]))
    with pytest.raises(MTGPError):
        pool.plan(work_items([0], [7], [10], [0]))


@pytest.mark.parametrize("bits,table", [(32, "mtgp32_fast_11213"), (64, "mtgp64dc_fast_11213"),
                                        (32, "mtgp32_fast_23209"), (64, "mtgp64_fast_23209")])
@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("core", [4, 2, 1])
@pytest.mark.parametrize("parts", [0, -1])
def test_batch_split_long_requests(gpu, orc, bits, table, mixed, core, parts):
    """Long requests split into chunks whose start states are GF(2) jumps,
    made ahead of the batched kernel by jump parts (parts 0: four CTAs per
    jump) or inside it (parts -1), on each 32-bit generation core: bit-exact
    outputs and final states, across two launches of the same plan."""
    from mtgp_gb300.api import Pool, work_items
    if bits == 64 and core == 4:
        pytest.skip("64-bit cores: two and one words per thread")
    tbl = load_table(table)
    rng = np.random.default_rng(bits + mixed + tbl[0].mexp)
    nstreams = 24
    plist = [tbl[i] for i in range(3)]
    pidx = np.arange(nstreams) % 3
    seeds = np.arange(nstreams) + 7
    pool = Pool.create(plist, seeds, pidx)
    counts = rng.integers(1, 30000, nstreams)
    counts[:4] = [1, 1499, 1875, 30001]
    kinds = rng.integers(0, 5, nstreams) if mixed else np.zeros(nstreams, np.int64)
    esz = bits // 8
    offs = np.concatenate([[0], np.cumsum(counts)[:-1]]) * esz
    # one stream gets two items (its run is cut across the item boundary)
    streams = list(range(nstreams)) + [5]
    kinds = list(kinds) + [0]
    counts = list(counts) + [20000]
    offs = list(offs) + [int(sum(counts[:-1])) * esz]
    pool.set_tuning("split_chunk", 1500)
    pool.set_tuning("core", core)
    pool.set_tuning("jump_parts", parts)
    plan = pool.plan(work_items(streams, kinds, counts, offs))
    ntasks, chunk = plan.info()
    assert chunk == 1500 and ntasks > nstreams
    desc = plan.describe()
    assert (desc["prejumps"] > 0 and not desc["jumps"]) if parts == 0 else \
        (desc["jumps"] and desc["prejumps"] == 0)
    out = torch.zeros(int(sum(counts)) * esz // 4 + 16, dtype=torch.int32, device="cuda")
    gens = {s: orc.gen(plist[pidx[s]], seed=int(seeds[s])) for s in range(nstreams)}
    for rep in range(2):
        plan.launch(out)
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(np.uint8)
        for k in range(len(streams)):
            ref = np_bits(gens[streams[k]].fill(int(kinds[k]), int(counts[k])), bits).view(np.uint8)
            assert np.array_equal(got[offs[k]:offs[k] + ref.size], ref), (rep, k)
        w = pool.windows()
        for s in range(nstreams):
            assert np.array_equal(w[s], gens[s].window()), (rep, s)


def test_batch_split_graph(gpu, orc):
    """The split plan (batched kernel + staged-window copy) replays from a
    CUDA graph."""
    from mtgp_gb300.api import Pool, work_items
    p = load_table("mtgp32_fast_11213")[0]
    pool = Pool.substreams(p, 1234, 16, jump_table(32))
    counts = np.array([100000, 5, 70000, 4096] + [3000] * 12)
    offs = np.concatenate([[0], np.cumsum(counts)[:-1]]) * 4
    pool.set_tuning("split_chunk", 16384)
    plan = pool.plan(work_items(np.arange(16), np.zeros(16), counts, offs))
    assert plan.info()[1] == 16384
    start = pool.windows()
    out = torch.zeros(int(counts.sum()), dtype=torch.int32, device="cuda")
    s = torch.cuda.Stream()
    gens = []
    for j in range(16):
        o = orc.gen(p, seed=1234)
        o.set_window(start[j])
        gens.append(o)
    for rep in range(3):
        plan.graph_launch(out, s)
        s.synchronize()
        got = out.cpu().numpy().view(np.uint32)
        for j in range(16):
            a = int(offs[j]) // 4
            assert np.array_equal(got[a:a + int(counts[j])], gens[j].fill(0, int(counts[j]))), (rep, j)


def test_autotune_leaves_pool_and_picks_exact_plan(gpu, orc):
    """The autotuner times candidates on the real items, restores the
    windows, and returns a plan whose output is bit-exact."""
    from mtgp_gb300.api import Pool, work_items
    p = load_table("mtgp32_fast_11213")[0]
    pool = Pool.substreams(p, 1234, 64, jump_table(32))
    rng = np.random.default_rng(5)
    counts = rng.integers(1000, 400000, 64)
    counts[0] = 1 << 20  # long enough to make split candidates real
    offs = np.concatenate([[0], np.cumsum(counts)[:-1]]) * 4
    items = work_items(np.arange(64), np.zeros(64), counts, offs)
    out = torch.zeros(int(counts.sum()), dtype=torch.int32, device="cuda")
    before = pool.windows()
    plan, report = pool.autotune(items, out, reps=1)
    assert np.array_equal(pool.windows(), before)
    assert report.count("ms") >= 3, report
    plan.launch(out)
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint32)
    for j in (0, 1, 37, 63):
        o = orc.gen(p, seed=1234)
        o.set_window(before[j])
        a = int(offs[j]) // 4
        assert np.array_equal(got[a:a + int(counts[j])], o.fill(0, int(counts[j]))), j


@pytest.mark.parametrize("bits,table", [(32, "mtgp32_fast_11213"), (64, "mtgp64dc_fast_11213"),
                                        (32, "mtgp32_fast_44497")])
@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("parts", [0, -1])
def test_batch_skip_then_split_chunks(gpu, orc, bits, table, mixed, parts):
    """Long requests that start after a long skip and are split into chunks:
    each chunk's start is the run start (a jump by the skip) then the chunk
    offset (a second jump).  Ahead of the launch (parts 0) the run starts
    are jumped once per run into middle slots and the chunk offsets from
    there, by a second launch of jump parts; inside the kernel (parts -1,
    where the exponent has it) the two jumps follow each other.  Bit-exact
    outputs and final states, across two launches of the same plan."""
    from mtgp_gb300.api import Pool, work_items
    tbl = load_table(table)
    if parts < 0 and tbl[0].mexp == 44497:
        pytest.skip("MEXP 44497 jumps only ahead of the launch")
    rng = np.random.default_rng(bits + 2 * mixed + tbl[0].mexp)
    nstreams = 12
    plist = [tbl[i] for i in range(3)]
    pidx = np.arange(nstreams) % 3
    seeds = np.arange(nstreams) + 11
    pool = Pool.create(plist, seeds, pidx)
    counts = rng.integers(2000, 9000, nstreams)
    skips = np.array([(1 << 17) + 12345, 1 << 20, 0, (1 << 18) + 3] * 3, np.uint64)
    kinds = rng.integers(0, 5, nstreams) if mixed else np.zeros(nstreams, np.int64)
    esz = bits // 8
    offs = np.concatenate([[0], np.cumsum(counts)[:-1]]) * esz
    pool.set_tuning("split_chunk", 1500)
    pool.set_tuning("jump_parts", parts)
    plan = pool.plan(work_items(range(nstreams), kinds, counts, offs, skips))
    desc = plan.describe()
    assert (desc["prejumps"] > nstreams and not desc["jumps"]) if parts == 0 else desc["jumps"]
    out = torch.zeros(int(sum(counts)) * esz // 4 + 16, dtype=torch.int32, device="cuda")
    gens = {s: orc.gen(plist[pidx[s]], seed=int(seeds[s])) for s in range(nstreams)}
    for rep in range(2):
        plan.launch(out)
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(np.uint8)
        for k in range(nstreams):
            gens[k].skip(int(skips[k]))
            ref = np_bits(gens[k].fill(int(kinds[k]), int(counts[k])), bits).view(np.uint8)
            assert np.array_equal(got[offs[k]:offs[k] + ref.size], ref), (rep, k)
        w = pool.windows()
        for s in range(nstreams):
            assert np.array_equal(w[s], gens[s].window()), (rep, s)


@pytest.mark.parametrize("bits,core", [(32, 4), (32, 2), (64, 2), (64, 1)])
@pytest.mark.parametrize("kind", [0, 1, 2, 3, 4, -1])
def test_batch_vector_cores_one_kind(gpu, orc, bits, core, kind):
    """The vector cores (32-bit: two and four words per thread; 64-bit: two,
    and the one-word core beside it) on plans of one output kind (no split):
    uneven counts, outputs at every word alignment (the cores' alignment
    pre-step), a skip item, against the oracle."""
    from mtgp_gb300.api import Pool, work_items
    tbl = load_table("mtgp32_fast_11213" if bits == 32 else "mtgp64dc_fast_11213")
    esz = bits // 8
    nstreams = 20
    plist = [tbl[i] for i in range(4)]
    pidx = np.arange(nstreams) % 4
    seeds = np.arange(nstreams) + 31
    pool = Pool.create(plist, seeds, pidx)
    rng = np.random.default_rng(core * 10 + kind + bits)
    counts = rng.integers(1, 9000, nstreams)
    counts[:5] = [1, 2, 3, 255, 4097]
    # consecutive outputs; each item starts 0..3 words after the previous one
    gaps = rng.integers(0, 4, nstreams)
    offs = np.zeros(nstreams, np.int64)
    pos = 0
    for k in range(nstreams):
        pos += int(gaps[k])
        offs[k] = pos * esz
        if kind >= 0:
            pos += int(counts[k])
    pool.set_tuning("core", core)
    pool.set_tuning("split_chunk", -1)
    plan = pool.plan(work_items(np.arange(nstreams), np.full(nstreams, kind), counts, offs))
    assert plan.describe()["core"] == core
    out = torch.zeros(pos * esz // 4 + 8, dtype=torch.int32, device="cuda")
    plan.launch(out)
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint8)
    for k in range(nstreams):
        o = orc.gen(plist[pidx[k]], seed=int(seeds[k]))
        ref = np_bits(o.fill(max(kind, 0), int(counts[k])), bits).view(np.uint8)
        if kind >= 0:
            assert np.array_equal(got[offs[k]:offs[k] + ref.size], ref), k
        assert np.array_equal(pool.windows()[k], o.window()), k


@pytest.mark.parametrize("bits,table", [(32, "mtgp32_fast_44497"), (64, "mtgp64_fast_44497"),
                                        (64, "mtgp64_fast_110503")])
def test_batch_jumps_made_ahead_for_large_exponents(gpu, orc, bits, table):
    """Exponents without the in-kernel jump still split long requests and
    jump long skips in a batch: every jumped start (a run start and a chunk
    offset combined into one polynomial made on the GPU) is made ahead of
    the launch by jump parts.  Outputs and windows (word 0 under the mask)
    against the oracle, which steps through the skips."""
    from mtgp_gb300.api import Pool, work_items
    tbl = load_table(table)
    p = tbl[0]
    nstreams = 4
    plist = [tbl[i % len(tbl)] for i in range(2)]
    pidx = np.arange(nstreams) % 2
    seeds = np.arange(nstreams) + 91
    pool = Pool.create(plist, seeds, pidx)
    jmin = 1 << 21 if p.mexp == 44497 else 1 << 24      # the planner's shortest jump
    pool.set_tuning("split_chunk", jmin)
    esz = bits // 8
    #        stream count             skip
    spec = [(0, 2 * jmin + 777, 0),                       # split: offsets only
            (1, 5000, jmin + 5),                          # one jumped skip
            (2, jmin + 3000, jmin),                       # run start + offset, combined
            (3, 4000, 0)]
    offs, pos = [], 0
    for _, c, _ in spec:
        offs.append(pos)
        pos += c * esz
    items = work_items([x[0] for x in spec], np.zeros(len(spec)), [x[1] for x in spec], offs,
                       [x[2] for x in spec])
    plan = pool.plan(items)
    desc = plan.describe()
    assert desc["prejumps"] >= 3 and not desc["jumps"], desc
    out = torch.zeros(pos // 4 + 16, dtype=torch.int32, device="cuda")
    plan.launch(out)
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint8)
    w = pool.windows()
    for (s, c, sk), off in zip(spec, offs):
        o = orc.gen(plist[pidx[s]], seed=int(seeds[s]))
        o.skip(sk)
        ref = np_bits(o.fill(0, c), bits).view(np.uint8)
        assert np.array_equal(got[off:off + ref.size], ref), s
        ow = o.window()
        assert (int(ow[0]) ^ int(w[s][0])) & int(plist[pidx[s]].mask) == 0, s
        assert np.array_equal(ow[1:], w[s][1:]), s
