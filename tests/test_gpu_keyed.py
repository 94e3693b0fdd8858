"""Key-schedule seeding on the device (init_by_array / init_by_str, one
thread per stream): pools of many streams with different parameter sets and
keys, against the oracle's windows and outputs."""
import numpy as np
import pytest
import torch

from mtgp_gb300.params import load_table
from gpu_util import as_np_bits

pytestmark = pytest.mark.gpu


def _keys(rng, bits, n):
    hi = 2 ** 32 if bits == 32 else 2 ** 63
    lens = [0, 1, 4, 350, 351, 352, 1000, 3000] + [int(x) for x in rng.integers(0, 800, n - 8)]
    return [rng.integers(0, hi, k, dtype=np.uint64) for k in lens[:n]]


@pytest.mark.parametrize("bits,table", [(32, "mtgp32_fast_11213"), (64, "mtgp64dc_fast_11213"),
                                        (32, "mtgp32_fast_23209"), (32, "mtgp32_fast_44497"),
                                        (64, "mtgp64_fast_44497")])
def test_pool_by_array(gpu, orc, bits, table):
    from mtgp_gb300.api import Pool
    tbl = load_table(table)
    plist = [tbl[i] for i in range(min(3, len(tbl)))]
    rng = np.random.default_rng(bits + len(plist))
    n = 24
    keys = _keys(rng, bits, n)
    if bits == 32:
        keys = [k.astype(np.uint32) for k in keys]
    pidx = np.arange(n) % len(plist)
    pool = Pool.create_by_array(plist, keys, pidx)
    win = pool.windows()
    for i in range(n):
        o = orc.gen(plist[pidx[i]], array=[int(x) for x in keys[i]])
        assert np.array_equal(win[i], o.window()), i
    # the streams continue like the reference's
    cnt = 3000
    dt = torch.int32 if bits == 32 else torch.int64
    out = torch.empty(n * cnt, dtype=dt, device="cuda")
    pool.fill(0, out, cnt)
    torch.cuda.synchronize()
    got = as_np_bits(out, bits).reshape(n, cnt)
    for i in (0, 5, n - 1):
        o = orc.gen(plist[pidx[i]], array=[int(x) for x in keys[i]])
        assert np.array_equal(got[i], o.fill(0, cnt)), i


@pytest.mark.parametrize("bits,table", [(32, "mtgp32_fast_11213"), (64, "mtgp64dc_fast_11213")])
def test_pool_by_str(gpu, orc, bits, table):
    from mtgp_gb300.api import Pool
    tbl = load_table(table)
    plist = [tbl[0], tbl[1]]
    strs = [b"", b"\x01\x02\x03\x04", b"\x80\xffhigh bytes", b"seed", b"x" * 500,
            bytes(range(1, 256))]
    pidx = [k % 2 for k in range(len(strs))]
    pool = Pool.create_by_str(plist, strs, pidx)
    win = pool.windows()
    for i, s in enumerate(strs):
        o = orc.gen(plist[pidx[i]], string=s)
        assert np.array_equal(win[i], o.window()), s


def test_keyed_pool_rejects_bad_offsets(gpu):
    import ctypes
    from mtgp_gb300._lib import lib
    from mtgp_gb300.params import MTGP32Params
    p = load_table("mtgp32_fast_11213")[0]
    arr = (MTGP32Params * 1)(p)
    keys = np.arange(8, dtype=np.uint32)
    off = np.array([0, 5, 3], dtype=np.uint64)   # decreasing
    h = ctypes.c_void_p()
    rc = lib().mtgp32_gpu_pool_create_by_array(
        ctypes.byref(h), arr, 1, None, keys.ctypes.data_as(ctypes.c_void_p),
        off.ctypes.data_as(ctypes.c_void_p), 2)
    assert rc != 0 and not h.value
