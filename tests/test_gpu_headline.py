"""The batched workload the throughput is quoted on, at full size.

MTGP32-11213 parameter set 0 (mtgp32_params_fast_11213[0]), seed 1234,
4096 substreams, substream j starting j * 3^162 steps ahead (made on the
GPU from the reference's jump table), and per substream one request of
lognormal length (median 2^16 uint32, sigma 1.0, seed 42, clipped to
[2^10, 2^22]): about 433 M values per launch.  The plan is the autotuner's,
launched twice from a CUDA graph.  Every substream's start window is checked
against the reference's own jump (JUMP3_162 applied j times), and every
output word of every substream and every final window against the oracle
(OpenMP over substreams), after each launch -- as the reference's own GPU
check compares every word and state (cuda-sample/mtgp32-sample-jump1-host.cu
9-128; word 0 of a state under the mask, :100-108).
"""
import numpy as np
import pytest
import torch

from mtgp_gb300.params import MTGP32Params, jump_string, jump_table, load_table, params_array

pytestmark = pytest.mark.gpu

N_SUB = 4096


def lengths(n=N_SUB, seed=42):
    rng = np.random.default_rng(seed)
    x = rng.lognormal(mean=np.log(2.0 ** 16), sigma=1.0, size=n)
    return np.clip(np.rint(x), 2 ** 10, 2 ** 22).astype(np.int64)


def _masked_equal_rows(a, b, mask):
    w0 = ((a[:, 0] ^ b[:, 0]) & np.uint32(mask)) == 0
    return w0 & (a[:, 1:] == b[:, 1:]).all(axis=1)


def test_lognormal_4096_substreams_full_size(gpu, orc):
    from mtgp_gb300.api import Pool, work_items
    p = load_table("mtgp32_fast_11213")[0]
    s = torch.cuda.Stream()
    pool = Pool.substreams(p, 1234, N_SUB, jump_table(32), stream=s)
    s.synchronize()
    start = pool.windows()
    # substream starts: the reference's jump by X^(3^162) applied j times
    o = orc.gen(p, seed=1234)
    js = jump_string(32)
    ref_start = np.empty_like(start)
    for j in range(N_SUB):
        ref_start[j] = o.window()
        o.fast_jump(js)
    ok = _masked_equal_rows(start, ref_start, p.mask)
    assert ok.all(), np.flatnonzero(~ok)[:10]

    lens = lengths()
    offs = np.concatenate([[0], np.cumsum(lens)[:-1]]) * 4
    items = work_items(np.arange(N_SUB), np.zeros(N_SUB), lens, offs)
    out = torch.empty(int(lens.sum()), dtype=torch.int32, device="cuda")
    plan, report = pool.autotune(items, out, stream=s, reps=3)
    assert np.array_equal(pool.windows(), start), "the autotuner must leave the windows"
    desc = plan.describe()
    parr = params_array(MTGP32Params, [p])
    win = np.ascontiguousarray(start.copy())
    ref = np.empty(int(lens.sum()), dtype=np.uint32)
    zeros = np.zeros(N_SUB, np.int32)
    for rep in range(2):
        out.fill_(-1)
        plan.graph_launch(out, s)
        s.synchronize()
        got = out.cpu().numpy().view(np.uint32)
        orc.multi_fill(32, parr, win, lens.astype(np.uint64), zeros, offs.astype(np.uint64), ref,
                       param_idx=zeros)
        if not np.array_equal(got, ref):
            bad = [j for j in range(N_SUB)
                   if not np.array_equal(got[offs[j] // 4:offs[j] // 4 + lens[j]],
                                         ref[offs[j] // 4:offs[j] // 4 + lens[j]])]
            pytest.fail("launch %d (%s): %d substreams differ, first %s"
                        % (rep, desc, len(bad), bad[:8]))
        ok = _masked_equal_rows(pool.windows(), win, p.mask)
        assert ok.all(), (rep, np.flatnonzero(~ok)[:10])
