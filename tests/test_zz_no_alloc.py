"""The allocation-free batched entry point (mtgp32_gpu_batch_noalloc).

It serves callers that cannot allocate device memory: engines whose device
memory is all reserved up front or under a hard budget, and plug-ins that may
only use buffers handed to them.  They pass their own window and output
buffers, and the library keeps the kernel's descriptors in a fixed device
array.  These tests call it through the C ABI twice in a row and check each
call's output and advanced windows bit-exactly against the pool entry point
(mtgp32_gpu_pool_submit) run on the same windows and items: batches of one
output kind (the two-word core), batches that mix kinds and advance-only
items (the one-word core), another exponent, and the default parameter
index; and batches with advance-only items directly against the oracle.
The file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest
import torch

from mtgp_gb300.params import MTGP32Params, load_table

pytestmark = pytest.mark.gpu


def _stride(mexp):
    return ((mexp // 32 + 1) + 31) // 32 * 32


def _items(rng, nstreams, nitems, kinds):
    from mtgp_gb300.api import work_items
    streams = rng.integers(0, nstreams, nitems)
    kind = rng.choice(np.asarray(kinds), nitems)
    counts = rng.integers(0, 9000, nitems)
    # advance-only items (kind -1) write nothing
    offs = np.concatenate([[0], np.cumsum(np.where(kind >= 0, counts, 0))[:-1]]) * 4
    total = int(np.where(kind >= 0, counts, 0).sum())
    return work_items(streams, kind, counts, offs), total


def _compare(table, nparams, nstreams, kinds, use_pidx, seed0):
    from mtgp_gb300._lib import check, lib
    from mtgp_gb300.api import Pool
    tbl = load_table(table)
    mexp = tbl[0].mexp
    size, stride = mexp // 32 + 1, _stride(mexp)
    plist = [tbl[i] for i in range(nparams)]
    if use_pidx:
        pidx = (np.arange(nstreams) % nparams).astype(np.int32)
    else:
        # without param_idx stream s uses set s (nparams == nstreams) or set 0
        pidx = (np.arange(nstreams) if nparams == nstreams
                else np.zeros(nstreams)).astype(np.int32)
    pool = Pool.create(plist, np.arange(nstreams) + seed0, pidx)
    # the caller-owned windows: same start states as the pool's
    win = np.zeros((nstreams, stride), dtype=np.uint32)
    win[:, :size] = pool.windows()
    dev_win = torch.from_numpy(win.view(np.int32)).cuda()
    parr = (MTGP32Params * nparams)(*plist)
    pptr = pidx.ctypes.data_as(ctypes.c_void_p) if use_pidx else None
    rng = np.random.default_rng(seed0)
    for call in range(2):
        items, total = _items(rng, nstreams, 150, kinds)
        ref = torch.zeros(total + 8, dtype=torch.int32, device="cuda")
        got = torch.zeros(total + 8, dtype=torch.int32, device="cuda")
        pool.submit(items, ref)
        stream = torch.cuda.current_stream()
        check(lib().mtgp32_gpu_batch_noalloc(
            parr, nparams, pptr, ctypes.c_void_p(dev_win.data_ptr()), nstreams, items,
            len(items), ctypes.c_void_p(got.data_ptr()), ctypes.c_void_p(stream.cuda_stream)))
        torch.cuda.synchronize()
        assert torch.equal(got, ref), call
        w = dev_win.cpu().numpy().view(np.uint32)[:, :size]
        assert np.array_equal(w, pool.windows()), call


def test_noalloc_vs_oracle(gpu, orc):
    """The entry point against the oracle directly: three parameter sets, a
    few streams, items of every output kind and advance-only items (the
    entry point takes no skips), in stream order, over two calls."""
    from mtgp_gb300._lib import check, lib
    from mtgp_gb300.api import Pool, work_items
    tbl = load_table("mtgp32_fast_11213")
    mexp = tbl[0].mexp
    size, stride = mexp // 32 + 1, _stride(mexp)
    nparams, nstreams = 3, 6
    plist = [tbl[i] for i in range(nparams)]
    pidx = (np.arange(nstreams) % nparams).astype(np.int32)
    seeds = np.arange(nstreams) + 77
    pool = Pool.create(plist, seeds, pidx)
    win = np.zeros((nstreams, stride), dtype=np.uint32)
    win[:, :size] = pool.windows()
    dev_win = torch.from_numpy(win.view(np.int32)).cuda()
    parr = (MTGP32Params * nparams)(*plist)
    gens = [orc.gen(plist[pidx[s]], seed=int(seeds[s])) for s in range(nstreams)]
    rng = np.random.default_rng(78)
    for call in range(2):
        n = 24
        streams = rng.integers(0, nstreams, n)
        kinds = rng.integers(-1, 5, n)
        counts = rng.integers(1, 7000, n)
        sizes = np.where(kinds >= 0, counts, 0)
        offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]) * 4
        items = work_items(streams, kinds, counts, offs)
        got = torch.zeros(int(sizes.sum()) + 8, dtype=torch.int32, device="cuda")
        check(lib().mtgp32_gpu_batch_noalloc(
            parr, nparams, pidx.ctypes.data_as(ctypes.c_void_p),
            ctypes.c_void_p(dev_win.data_ptr()), nstreams, items, n,
            ctypes.c_void_p(got.data_ptr()),
            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
        torch.cuda.synchronize()
        out = got.cpu().numpy().view(np.uint8)
        for k in range(n):
            g = gens[streams[k]]
            if kinds[k] < 0:
                g.skip(int(counts[k]))
                continue
            ref = np.ascontiguousarray(g.fill(int(kinds[k]), int(counts[k]))).view(np.uint8)
            assert np.array_equal(out[offs[k]:offs[k] + ref.size], ref), (call, k)
        w = dev_win.cpu().numpy().view(np.uint32)[:, :size]
        for s in range(nstreams):
            assert np.array_equal(w[s], gens[s].window()), (call, s)


@pytest.mark.parametrize("kinds", [[0], [3], [0, 1, 2, 3, 4], [-1, 0, 2]],
                         ids=["uint32", "open_close", "mixed", "mixed_advance"])
def test_noalloc_matches_pool_submit_twice(gpu, kinds):
    _compare("mtgp32_fast_11213", 3, 40, kinds, True, 501)


def test_noalloc_other_exponent_and_default_index(gpu):
    _compare("mtgp32_fast_23209", 4, 4, [0, 1], False, 901)
    _compare("mtgp32_fast_11213", 2, 12, [0], False, 77)


def test_noalloc_rejects_oversized_requests(gpu):
    from mtgp_gb300._lib import lib
    from mtgp_gb300.api import work_items
    tbl = load_table("mtgp32_fast_11213")
    dev_win = torch.zeros(4 * 352, dtype=torch.int32, device="cuda")
    out = torch.zeros(16, dtype=torch.int32, device="cuda")
    many = work_items(np.zeros(2049), np.zeros(2049), np.ones(2049), np.zeros(2049))
    parr = (MTGP32Params * 1)(tbl[0])
    rc = lib().mtgp32_gpu_batch_noalloc(parr, 1, None, ctypes.c_void_p(dev_win.data_ptr()), 4,
                                        many, len(many), ctypes.c_void_p(out.data_ptr()), None)
    assert rc == -2 and b"2048" in lib().mtgp_gpu_last_error()
    parr17 = (MTGP32Params * 17)(*[tbl[i] for i in range(17)])
    one = work_items([0], [0], [4], [0])
    rc = lib().mtgp32_gpu_batch_noalloc(parr17, 17, None, ctypes.c_void_p(dev_win.data_ptr()), 4,
                                        one, 1, ctypes.c_void_p(out.data_ptr()), None)
    assert rc == -2 and b"16" in lib().mtgp_gpu_last_error()


def test_noalloc_refuses_a_capturing_stream(gpu):
    """The call synchronises its stream, which a stream under capture does
    not allow: it returns MTGP_ERR_UNSUPPORTED and the caller's capture goes
    on unharmed."""
    from mtgp_gb300._lib import lib
    from mtgp_gb300.api import work_items
    tbl = load_table("mtgp32_fast_11213")
    dev_win = torch.zeros(4 * 352, dtype=torch.int32, device="cuda")
    out = torch.zeros(16, dtype=torch.int32, device="cuda")
    x = torch.zeros(8, device="cuda")
    parr = (MTGP32Params * 1)(tbl[0])
    one = work_items([0], [0], [4], [0])
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        x += 1
        rc = lib().mtgp32_gpu_batch_noalloc(
            parr, 1, None, ctypes.c_void_p(dev_win.data_ptr()), 4, one, 1,
            ctypes.c_void_p(out.data_ptr()),
            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == -3 and b"captured" in lib().mtgp_gpu_last_error()
    g.replay()
    torch.cuda.synchronize()
    assert float(x[0]) == 1.0
