"""Parameter sets and jump tables of the MTGP reference, as ctypes structs.

The structs have the reference's exact layout (mtgp32-fast.h:47-58 and
mtgp64-fast.h:46-57), so a pointer to one element can be passed straight to
the C ABI (include/mtgp_gpu.h) or to the reference library.

Tables (files in mtgp_gb300/data, exported from the reference sources by
data/make_tables.py):

==========================  =====  ==========================================
name                        count  reference symbol (file)
==========================  =====  ==========================================
mtgp32_fast_11213            128   mtgp32_params_fast_11213 (mtgp32-param-fast.c:4)
mtgp32_fast_23209            128   mtgp32_params_fast_23209 (mtgp32-param-fast.c:7432)
mtgp32_fast_44497            128   mtgp32_params_fast_44497 (mtgp32-param-fast.c:14860)
mtgp32dc_fast_11213          200   mtgp32dc_params_fast_11213 (cuda-sample/mtgp32dc-param-11213.c:4)
mtgp64_fast_23209            128   mtgp64_params_fast_23209 (mtgp64-param-fast.c:4)
mtgp64_fast_44497            128   mtgp64_params_fast_44497 (mtgp64-param-fast.c:7432)
mtgp64_fast_110503           128   mtgp64_params_fast_110503 (mtgp64-param-fast.c:14860)
mtgp64dc_fast_11213          200   mtgp64dc_params_fast_11213 (openCL-sample/mtgp64dc-param-11213.c:9)
mtgp64dc_cuda_fast_11213     200   mtgp64dc_params_fast_11213 (cuda-sample/mtgp64dc-param-11213.c:9)
==========================  =====  ==========================================
"""
import ctypes
import os

import numpy as np

DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")


class MTGP32Params(ctypes.Structure):
    """mtgp32_params_fast_t (mtgp32-fast.h:47-58)."""
    _fields_ = [("mexp", ctypes.c_int), ("pos", ctypes.c_int),
                ("sh1", ctypes.c_int), ("sh2", ctypes.c_int),
                ("tbl", ctypes.c_uint32 * 16), ("tmp_tbl", ctypes.c_uint32 * 16),
                ("flt_tmp_tbl", ctypes.c_uint32 * 16), ("mask", ctypes.c_uint32),
                ("poly_sha1", ctypes.c_ubyte * 21)]


class MTGP64Params(ctypes.Structure):
    """mtgp64_params_fast_t (mtgp64-fast.h:46-57)."""
    _fields_ = [("mexp", ctypes.c_int), ("pos", ctypes.c_int),
                ("sh1", ctypes.c_int), ("sh2", ctypes.c_int),
                ("tbl", ctypes.c_uint64 * 16), ("tmp_tbl", ctypes.c_uint64 * 16),
                ("dbl_tmp_tbl", ctypes.c_uint64 * 16), ("mask", ctypes.c_uint64),
                ("poly_sha1", ctypes.c_ubyte * 21)]


assert ctypes.sizeof(MTGP32Params) == 236
assert ctypes.sizeof(MTGP64Params) == 432

TABLES = {
    "mtgp32_fast_11213": (32, 128), "mtgp32_fast_23209": (32, 128),
    "mtgp32_fast_44497": (32, 128), "mtgp32dc_fast_11213": (32, 200),
    "mtgp64_fast_23209": (64, 128), "mtgp64_fast_44497": (64, 128),
    "mtgp64_fast_110503": (64, 128), "mtgp64dc_fast_11213": (64, 200),
    "mtgp64dc_cuda_fast_11213": (64, 200),
}

_cache = {}


def load_table(name):
    """Return the named table as a ctypes array of MTGP32Params/MTGP64Params."""
    if name in _cache:
        return _cache[name]
    bits, count = TABLES[name]
    cls = MTGP32Params if bits == 32 else MTGP64Params
    with open(os.path.join(DATA, name + ".bin"), "rb") as f:
        raw = f.read()
    if len(raw) != count * ctypes.sizeof(cls):
        raise ValueError("table %s has %d bytes, expected %d"
                         % (name, len(raw), count * ctypes.sizeof(cls)))
    arr = (cls * count).from_buffer_copy(raw)
    _cache[name] = arr
    return arr


def params_array(cls, items):
    """Pack a list of parameter structs into one contiguous ctypes array."""
    arr = (cls * len(items))()
    for k, p in enumerate(items):
        arr[k] = p
    return arr


def jump_table(bits):
    """The shipped long-jump table for set 0 of the 11213 tables: row k is
    X^(4^k * 3^162) mod chi in the uint32-array form (k = 0..5), 351 words.

    32-bit: openCL-sample/mtgp32-jump-table.cpp (== cuda-sample/
    mtgp32-jump-table.h rows[:351]) for mtgp32_params_fast_11213[0];
    64-bit: openCL-sample/mtgp64-jump-table.cpp for the OpenCL
    mtgp64dc_params_fast_11213[0]."""
    path = os.path.join(DATA, "mtgp%d_jump_11213.bin" % bits)
    return np.fromfile(path, dtype="<u4").reshape(6, 351)


def jump_string(bits):
    """X^(3^162) mod chi as the reference's hex string
    (openCL-sample/mtgp32-jump-string.h, mtgp64-jump-string.h)."""
    with open(os.path.join(DATA, "mtgp%d_jump3_162.txt" % bits)) as f:
        return f.read().strip()


def characteristic_string(bits):
    """Characteristic polynomial of set 0 (cuda-sample/mtgp32-char11213.h,
    openCL-sample/characteristic.64.11213.txt) in hex form."""
    with open(os.path.join(DATA, "mtgp%d_char_11213.txt" % bits)) as f:
        return f.read().strip()


def state_size(p):
    """Live state words: mexp / word_bits + 1 (mtgp32-fast.c:36-58)."""
    return p.mexp // (32 if isinstance(p, MTGP32Params) else 64) + 1
