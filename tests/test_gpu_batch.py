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
