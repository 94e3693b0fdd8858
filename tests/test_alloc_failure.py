"""Allocation failure: the reference's -1 path (mtgp32-fast.c:47-51).

The library routes every device and pinned host allocation through one
wrapper; MTGP_TEST_FAIL_ALLOC=k in the environment makes allocation number k
of the process fail as an out-of-memory error, on the host, without touching
the GPU.  Each case runs in a child process (the variable is read once).  A
failed create must return MTGP_ERR_ALLOC (-1), leave the output handle NULL
and free what it had already allocated.
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import ctypes, json, sys
import numpy as np
sys.path.insert(0, %(root)r)
from mtgp_gb300._lib import lib
from mtgp_gb300.params import load_table, MTGP32Params
L = lib()
p = load_table("mtgp32_fast_11213")[0]
what, count, gpu = sys.argv[1], int(sys.argv[2]), sys.argv[3] == "1"
free0 = None
if gpu:
    import torch
    torch.cuda.init()
    free0 = torch.cuda.mem_get_info()[0]
h = ctypes.c_void_p()
if what == "pool":
    seeds = np.arange(count, dtype=np.uint32)
    rc = L.mtgp32_gpu_pool_create(ctypes.byref(h), ctypes.byref(p), 1, None,
                                  seeds.ctypes.data_as(ctypes.c_void_p), count)
else:
    rc = L.mtgp32_gpu_init(ctypes.byref(h), ctypes.byref(p), 1234)
out = {"rc": rc, "handle_null": not h.value, "msg": L.mtgp_gpu_last_error().decode()}
if gpu:
    torch.cuda.synchronize()
    out["leaked"] = free0 - torch.cuda.mem_get_info()[0]
    if h.value:
        (L.mtgp32_gpu_pool_free if what == "pool" else L.mtgp32_gpu_free)(h)
print(json.dumps(out))
"""


def _child(k, what, count, gpu):
    env = dict(os.environ, MTGP_TEST_FAIL_ALLOC=str(k))
    r = subprocess.run([sys.executable, "-c", CHILD % {"root": ROOT}, what, str(count),
                        "1" if gpu else "0"], capture_output=True, text=True, env=env,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return json.loads(r.stdout.strip().splitlines()[-1])


@pytest.mark.parametrize("what", ["pool", "gen"])
def test_first_allocation_failure_returns_alloc_error(what):
    """Allocation 0 (the parameter sets) fails before any CUDA call, so this
    runs without a GPU."""
    from mtgp_gb300 import build as b
    b.build()
    out = _child(0, what, 16, False)
    assert out["rc"] == -1 and out["handle_null"], out
    assert "out of memory" in out["msg"] or "memory" in out["msg"], out


@pytest.mark.gpu
@pytest.mark.parametrize("what", ["pool", "gen"])
def test_allocation_failures_leak_nothing(gpu, what):
    """Every allocation of a create fails in turn (parameter sets, parameter
    indices, the windows of 2^19 streams = 738 MB, the seeds): each returns
    MTGP_ERR_ALLOC with a NULL handle, and the device memory it had taken is
    given back; with no failure injected the same create succeeds."""
    count = 1 << 19 if what == "pool" else 1
    for k in range(4):
        out = _child(k, what, count, True)
        assert out["rc"] == -1 and out["handle_null"], (k, out)
        assert out["leaked"] < 64 << 20, (k, out)
    out = _child(10 ** 6, what, count, True)
    assert out["rc"] == 0 and not out["handle_null"], out
