"""The allocation-free batched entry point (mtgp32_gpu_batch_noalloc).

It serves callers that cannot allocate device memory: engines whose device
memory is all reserved up front or under a hard budget, and plug-ins that may
only use buffers handed to them.  They pass their own window and output
buffers, and the library keeps the kernel's descriptors in a fixed device
array.  This test calls it through the C ABI twice in a row and checks each
call's output and advanced windows bit-exactly against the pool entry point
(mtgp32_gpu_pool_submit) run on the same windows and items.  The file is
named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest
import torch

from mtgp_gb300.params import MTGP32Params, load_table

pytestmark = pytest.mark.gpu

STRIDE = 352  # roundup(11213/32 + 1, 32) words per window


def _items(rng, nstreams, nitems):
    from mtgp_gb300.api import work_items
    streams = rng.integers(0, nstreams, nitems)
    kinds = rng.integers(0, 5, nitems)
    counts = rng.integers(0, 9000, nitems)
    offs = np.concatenate([[0], np.cumsum(counts)[:-1]]) * 4
    return work_items(streams, kinds, counts, offs), int(counts.sum())


def test_noalloc_matches_pool_submit_twice(gpu):
    from mtgp_gb300._lib import check, lib
    from mtgp_gb300.api import Pool
    tbl = load_table("mtgp32_fast_11213")
    nparams, nstreams = 3, 40
    plist = [tbl[i] for i in range(nparams)]
    pidx = (np.arange(nstreams) % nparams).astype(np.int32)
    seeds = np.arange(nstreams) + 501
    pool = Pool.create(plist, seeds, pidx)
    # the caller-owned windows: same start states as the pool's
    win = np.zeros((nstreams, STRIDE), dtype=np.uint32)
    win[:, :351] = pool.windows()
    dev_win = torch.from_numpy(win.view(np.int32)).cuda()
    parr = (MTGP32Params * nparams)(*plist)
    rng = np.random.default_rng(11)
    for call in range(2):
        items, total = _items(rng, nstreams, 150)
        ref = torch.zeros(total + 8, dtype=torch.int32, device="cuda")
        got = torch.zeros(total + 8, dtype=torch.int32, device="cuda")
        pool.submit(items, ref)
        stream = torch.cuda.current_stream()
        check(lib().mtgp32_gpu_batch_noalloc(
            parr, nparams, pidx.ctypes.data_as(ctypes.c_void_p),
            ctypes.c_void_p(dev_win.data_ptr()), nstreams, items, len(items),
            ctypes.c_void_p(got.data_ptr()), ctypes.c_void_p(stream.cuda_stream)))
        torch.cuda.synchronize()
        assert torch.equal(got, ref), call
        w = dev_win.cpu().numpy().view(np.uint32)[:, :351]
        assert np.array_equal(w, pool.windows()), call


def test_noalloc_rejects_oversized_requests(gpu):
    from mtgp_gb300._lib import lib
    from mtgp_gb300.api import work_items
    tbl = load_table("mtgp32_fast_11213")
    dev_win = torch.zeros(4 * STRIDE, dtype=torch.int32, device="cuda")
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
