"""Plain path on the GPU vs the oracle: every output bit-exact."""
import ctypes

import numpy as np
import pytest
import torch

from mtgp_gb300.params import load_table
from gpu_util import as_np_bits, check_guards, guarded, np_bits

pytestmark = pytest.mark.gpu

T32 = [("mtgp32_fast_11213", 0), ("mtgp32_fast_11213", 127), ("mtgp32dc_fast_11213", 17),
       ("mtgp32_fast_23209", 5), ("mtgp32_fast_44497", 9)]
T64 = [("mtgp64dc_fast_11213", 0), ("mtgp64dc_fast_11213", 199), ("mtgp64dc_cuda_fast_11213", 3),
       ("mtgp64_fast_23209", 1), ("mtgp64_fast_44497", 2), ("mtgp64_fast_110503", 4)]


def _gen(bits, p, **kw):
    from mtgp_gb300.api import MTGP32, MTGP64
    return (MTGP32 if bits == 32 else MTGP64)(p, **kw)


def _run(gen, kind, n, bits):
    full, view = guarded(n, bits, kind)
    gen.fill_into(kind, view, n)
    torch.cuda.synchronize()
    check_guards(full, bits)
    return as_np_bits(view, bits)


def test_config1_uint32_then_float(gpu, orc):
    """Set 0 of the 11213 table, seed 1234: 2^20 uint32 then 2^20 float [1,2)."""
    p = load_table("mtgp32_fast_11213")[0]
    g = _gen(32, p, seed=1234)
    o = orc.gen(p, seed=1234)
    n = 1 << 20
    assert np.array_equal(_run(g, 0, n, 32), o.fill(0, n))
    assert np.array_equal(_run(g, 1, n, 32), np_bits(o.fill(1, n), 32))
    assert np.array_equal(g.window(), o.window())


@pytest.mark.parametrize("bits,table,idx", [(32,) + t for t in T32] + [(64,) + t for t in T64])
@pytest.mark.parametrize("kind", [0, 1, 2, 3, 4])
def test_all_kinds_and_tables(gpu, orc, bits, table, idx, kind):
    p = load_table(table)[idx]
    g = _gen(bits, p, seed=4242 + idx)
    o = orc.gen(p, seed=4242 + idx)
    for n in (3000, 1, 4099):
        assert np.array_equal(_run(g, kind, n, bits), np_bits(o.fill(kind, n), bits)), n
    assert np.array_equal(g.window(), o.window())


@pytest.mark.parametrize("n", [1, 2, 127, 128, 129, 255, 256, 257, 351, 352, 767, 768, 769, 1000])
def test_ragged_counts_continue(gpu, orc, n):
    for bits, table in ((32, "mtgp32_fast_11213"), (64, "mtgp64dc_fast_11213")):
        p = load_table(table)[3]
        g = _gen(bits, p, seed=n)
        o = orc.gen(p, seed=n)
        for rep in range(3):
            assert np.array_equal(_run(g, 0, n, bits), o.fill(0, n)), (bits, n, rep)


def test_zero_count_is_noop(gpu, orc):
    p = load_table("mtgp32_fast_11213")[0]
    g = _gen(32, p, seed=5)
    o = orc.gen(p, seed=5)
    g.fill(0, 0)
    assert np.array_equal(_run(g, 0, 10, 32), o.fill(0, 10))


@pytest.mark.parametrize("bits,table", [(32, "mtgp32_fast_11213"), (64, "mtgp64dc_fast_11213")])
def test_init_by_array_and_str(gpu, orc, bits, table):
    p = load_table(table)[1]
    for kw in (dict(array=[1, 2, 3, 4]), dict(array=list(range(1000))), dict(array=[]),
               dict(string=b"\x01\x02\x03\x04"), dict(string=b"\x80\xffhigh bytes"),
               dict(string=b"")):
        g = _gen(bits, p, **kw)
        o = orc.gen(p, **kw)
        assert np.array_equal(g.window(), o.window()), kw
        assert np.array_equal(_run(g, 0, 2000, bits), o.fill(0, 2000)), kw


def test_skip_matches_stepping(gpu, orc):
    for bits, table in ((32, "mtgp32_fast_11213"), (64, "mtgp64dc_fast_11213")):
        p = load_table(table)[0]
        g = _gen(bits, p, seed=7)
        o = orc.gen(p, seed=7)
        for n in (1, 300, 100003, (1 << 22) + 5):   # the last one is a jump
            g.skip(n)
            o.skip(n)
            assert np.array_equal(_run(g, 0, 500, bits), o.fill(0, 500))


def test_export_import_roundtrip(gpu, orc):
    """The device state continues exactly in the reference struct layout."""
    from mtgp_gb300._lib import lib, check
    from mtgp_gb300.api import MTGP32
    p = load_table("mtgp32_fast_11213")[0]
    g = MTGP32(p, seed=99)
    g.fill(0, 12345)
    torch.cuda.synchronize()

    class Status(ctypes.Structure):
        _fields_ = [("idx", ctypes.c_int), ("size", ctypes.c_int), ("large_size", ctypes.c_int),
                    ("large_mask", ctypes.c_int), ("array", ctypes.c_uint32 * 512)]

    from mtgp_gb300.params import MTGP32Params

    class Fast(ctypes.Structure):
        _fields_ = [("params", MTGP32Params), ("status", ctypes.POINTER(Status))]

    st = Status(idx=0, size=351, large_size=512, large_mask=511)
    f = Fast(params=p, status=ctypes.pointer(st))
    check(lib().mtgp32_gpu_export(g.h, ctypes.byref(f)))
    o = orc.gen(p, seed=99)
    o.fill(0, 12345)
    win = np.array([st.array[(st.idx - 350 + k) % 512] for k in range(351)], dtype=np.uint32)
    assert np.array_equal(win, o.window())
    # rotate the ring so import must honour idx
    st2 = Status(idx=100, size=351, large_size=512, large_mask=511)
    for k in range(351):
        st2.array[(100 - 350 + k) % 512] = int(win[k])
    f2 = Fast(params=p, status=ctypes.pointer(st2))
    h2 = MTGP32(p, seed=1)
    check(lib().mtgp32_gpu_import(h2.h, ctypes.byref(f2)))
    assert np.array_equal(h2.fill(0, 5000).cpu().numpy().view(np.uint32), o.fill(0, 5000))


def test_errors_are_status_codes(gpu):
    from mtgp_gb300._lib import MTGPError
    from mtgp_gb300.api import MTGP32
    p = load_table("mtgp32_fast_11213")[0]
    g = MTGP32(p, seed=1)
    with pytest.raises(MTGPError) as e:
        g.fast_jump("12z4")
    assert e.value.code == -4
    bad = load_table("mtgp32_fast_11213")[0]
    import copy
    bad = copy.copy(bad)
    bad.mexp = 12345
    with pytest.raises(MTGPError) as e:
        MTGP32(bad, seed=1)
    assert e.value.code == -3
    out = torch.empty(8, dtype=torch.int32, device="cuda")
    from mtgp_gb300._lib import lib
    rc = lib().mtgp32_gpu_fill(g.h, 0, ctypes.c_void_p(out.data_ptr() + 2), 4, None)
    assert rc == -2
    rc = lib().mtgp32_gpu_fill(g.h, 9, ctypes.c_void_p(out.data_ptr()), 4, None)
    assert rc == -2
