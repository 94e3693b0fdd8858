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
