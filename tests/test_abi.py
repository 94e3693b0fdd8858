"""The C-ABI library loads and exports every function include/mtgp_gpu.h
declares (no GPU calls)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(mtgp\w*)\s*\(", src):
            names.add(m.group(1))
    return names


def test_header_declares_reference_api():
    names = declared_functions()
    for n in ("mtgp32_gpu_init", "mtgp32_gpu_init_by_array", "mtgp32_gpu_init_by_str",
              "mtgp32_gpu_fill_uint32", "mtgp32_gpu_fill_close1_open2",
              "mtgp32_gpu_fill_close_open", "mtgp32_gpu_fill_open_close",
              "mtgp32_gpu_fill_open_open", "mtgp32_gpu_fast_jump", "mtgp64_gpu_fast_jump",
              "mtgp64_gpu_fill_uint64", "mtgp32_gpu_free", "mtgp64_gpu_free"):
        assert n in names


def test_library_exports_every_declared_symbol():
    from mtgp_gb300 import build
    build.build()
    lib = ctypes.CDLL(build.LIB)
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header():
    from mtgp_gb300._lib import SIGS
    missing = sorted(declared_functions() - set(SIGS))
    assert not missing, missing


def test_struct_layouts_match_reference():
    from mtgp_gb300.params import MTGP32Params, MTGP64Params
    assert ctypes.sizeof(MTGP32Params) == 236
    assert ctypes.sizeof(MTGP64Params) == 432
    assert MTGP32Params.mask.offset == 208 and MTGP64Params.mask.offset == 400


def test_tuning_keys_and_ranges():
    """mtgp_gpu_set_tuning accepts the documented keys and values and
    rejects the rest (host-side settings only: no GPU call)."""
    from mtgp_gb300 import build
    build.build()
    lib = ctypes.CDLL(build.LIB)
    lib.mtgp_gpu_set_tuning.argtypes = [ctypes.c_char_p, ctypes.c_int64]
    lib.mtgp_gpu_set_tuning.restype = ctypes.c_int
    ok = [(b"split_chunk", 0), (b"split_chunk", -1), (b"split_chunk", 1 << 17),
          (b"batch_grid", 0), (b"batch_grid", 760), (b"core", 1), (b"core", 4), (b"core", 2),
          (b"poly_window", 2), (b"poly_window", 0), (b"single_chunk", 1 << 15),
          (b"single_chunk", 0), (b"jump_parts", -1), (b"jump_parts", 11), (b"jump_parts", 0)]
    bad = [(b"core", 3), (b"poly_window", 3), (b"batch_grid", -1), (b"single_chunk", -1),
           (b"jump_parts", -2), (b"no_such_knob", 0)]
    for k, v in ok:
        assert lib.mtgp_gpu_set_tuning(k, v) == 0, (k, v)
    for k, v in bad:
        assert lib.mtgp_gpu_set_tuning(k, v) == -2, (k, v)  # MTGP_ERR_INVALID
    # the defaults again: later tests in this process see a clean state
    for k, v in ((b"split_chunk", 0), (b"batch_grid", 0), (b"core", 2), (b"poly_window", 0),
                 (b"single_chunk", 0), (b"jump_parts", 0)):
        assert lib.mtgp_gpu_set_tuning(k, v) == 0
