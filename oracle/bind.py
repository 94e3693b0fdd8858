"""ctypes bindings for the test oracle.  TEST INFRASTRUCTURE ONLY.

`Oracle` wraps oracle/liboracle.so (our C restatement of the reference,
oracle/mtgp_oracle.c); `Reference` wraps oracle/_ref/libmtgpref.so (the
reference's own sources compiled in place), which exists only where the
reference tree is available.  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg use this module.
"""
import ctypes
import os
import subprocess

import numpy as np

from mtgp_gb300.params import MTGP32Params, MTGP64Params

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REFLIB = os.path.join(HERE, "_ref", "libmtgpref.so")

_P = ctypes.c_void_p
_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)


def build(ref=False):
    """Compile liboracle.so (and the reference library if ref=True)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])
    if ref:
        subprocess.check_call(["make", "-s", "-C", HERE, "ref"])


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    """CPU restatement; one instance per process is enough."""

    def __init__(self):
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        self.L = L
        for b, pt in ((32, MTGP32Params), (64, MTGP64Params)):
            pre = "orc%d_" % b
            wt = ctypes.c_uint32 if b == 32 else ctypes.c_uint64
            getattr(L, pre + "new_seed").restype = _P
            getattr(L, pre + "new_seed").argtypes = [ctypes.POINTER(pt), wt]
            getattr(L, pre + "new_array").restype = _P
            getattr(L, pre + "new_array").argtypes = [ctypes.POINTER(pt), _P, ctypes.c_int]
            getattr(L, pre + "new_str").restype = _P
            getattr(L, pre + "new_str").argtypes = [ctypes.POINTER(pt), ctypes.c_char_p]
            getattr(L, pre + "clone").restype = _P
            getattr(L, pre + "clone").argtypes = [_P]
            getattr(L, pre + "delete").argtypes = [_P]
            getattr(L, pre + "size").argtypes = [_P]
            getattr(L, pre + "fill").argtypes = [_P, ctypes.c_int, _P, ctypes.c_size_t]
            getattr(L, pre + "skip").argtypes = [_P, ctypes.c_uint64]
            getattr(L, pre + "fast_jump").argtypes = [_P, ctypes.c_char_p]
            getattr(L, pre + "jump_words").argtypes = [_P, _P, ctypes.c_int]
            getattr(L, pre + "get_window").argtypes = [_P, _P]
            getattr(L, pre + "set_window").argtypes = [_P, _P]
            getattr(L, pre + "get_ring").argtypes = [_P, _P]
            getattr(L, pre + "multi_fill").argtypes = [
                ctypes.POINTER(pt), ctypes.c_int, _P, _P, ctypes.c_int, _P, _P, _P,
                _P, ctypes.c_int]
            getattr(L, pre + "seed_windows").argtypes = [
                ctypes.POINTER(pt), _P, _P, ctypes.c_int, _P]
        L.orc_gf2_minpoly.argtypes = [_P, ctypes.c_int, _P, ctypes.c_int]
        L.orc_gf2_powxmod.argtypes = [_P, ctypes.c_int, _P, ctypes.c_int, _P]
        L.orc_gf2_mulmod.argtypes = [_P, _P, _P, ctypes.c_int, _P]
        L.orc_gf2_from_hex.argtypes = [ctypes.c_char_p, _P, ctypes.c_int]
        L.orc_gf2_to_hex.argtypes = [_P, ctypes.c_int, ctypes.c_char_p, ctypes.c_int]

    def max_threads(self):
        return self.L.orc_max_threads()

    def gen(self, params, seed=None, array=None, string=None):
        return OracleGen(self, params, seed, array, string)

    # ---- GF(2)[x] ----
    def minpoly(self, bits):
        bits = np.ascontiguousarray(bits, dtype=np.uint8)
        nw = len(bits) // 64 + 2
        out = np.zeros(nw, dtype=np.uint64)
        d = self.L.orc_gf2_minpoly(_ptr(bits), len(bits), _ptr(out), nw)
        return d, out

    def powxmod(self, e, m, dm):
        """X^e mod m; e a Python int, m uint64 words of degree dm."""
        ew = max(1, (e.bit_length() + 31) // 32)
        ea = np.array([(e >> (32 * k)) & 0xffffffff for k in range(ew)], dtype=np.uint32)
        out = np.zeros((dm + 63) // 64, dtype=np.uint64)
        m = np.ascontiguousarray(m, dtype=np.uint64)
        self.L.orc_gf2_powxmod(_ptr(ea), ew, _ptr(m), dm, _ptr(out))
        return out

    def mulmod(self, a, b, m, dm):
        out = np.zeros((dm + 63) // 64, dtype=np.uint64)
        self.L.orc_gf2_mulmod(_ptr(np.ascontiguousarray(a, np.uint64)),
                              _ptr(np.ascontiguousarray(b, np.uint64)),
                              _ptr(np.ascontiguousarray(m, np.uint64)), dm, _ptr(out))
        return out

    def from_hex(self, s, nwords):
        out = np.zeros(nwords, dtype=np.uint64)
        n = self.L.orc_gf2_from_hex(s.encode(), _ptr(out), nwords)
        if n < 0:
            raise ValueError("bad hex digit")
        return out

    def to_hex(self, p, degree):
        buf = ctypes.create_string_buffer(degree // 4 + 8)
        self.L.orc_gf2_to_hex(_ptr(np.ascontiguousarray(p, np.uint64)), degree, buf, len(buf))
        return buf.value.decode()

    # ---- many generators (OpenMP) ----
    def multi_fill(self, bits, params_arr, windows, counts, kinds, offsets, out,
                   param_idx=None, nthreads=0):
        pre = "orc%d_" % bits
        counts = np.ascontiguousarray(counts, np.uint64)
        kinds = np.ascontiguousarray(kinds, np.int32)
        offsets = np.ascontiguousarray(offsets, np.uint64)
        pidx = None if param_idx is None else np.ascontiguousarray(param_idx, np.int32)
        getattr(self.L, pre + "multi_fill")(
            params_arr, len(params_arr), None if pidx is None else _ptr(pidx),
            _ptr(windows), len(counts), _ptr(counts), _ptr(kinds), _ptr(offsets),
            _ptr(out), nthreads)

    def seed_windows(self, bits, params_arr, seeds, param_idx=None):
        size = params_arr[0].mexp // bits + 1
        n = len(seeds)
        dt = np.uint32 if bits == 32 else np.uint64
        seeds = np.ascontiguousarray(seeds, dt)
        win = np.zeros(n * size, dtype=dt)
        pidx = None if param_idx is None else np.ascontiguousarray(param_idx, np.int32)
        getattr(self.L, "orc%d_seed_windows" % bits)(
            params_arr, None if pidx is None else _ptr(pidx), _ptr(seeds), n, _ptr(win))
        return win.reshape(n, size)


class OracleGen:
    """One generator of the restatement (mirrors mtgp32_fast_t usage)."""

    def __init__(self, orc, params, seed=None, array=None, string=None, _h=None):
        self.o = orc
        self.bits = 32 if isinstance(params, MTGP32Params) else 64
        self.params = params
        self.pre = "orc%d_" % self.bits
        self.wdt = np.uint32 if self.bits == 32 else np.uint64
        L = orc.L
        if _h is not None:
            self.h = _h
        elif string is not None:
            self.h = getattr(L, self.pre + "new_str")(ctypes.byref(params), string)
        elif array is not None:
            a = np.ascontiguousarray(array, self.wdt)
            self._keep = a
            self.h = getattr(L, self.pre + "new_array")(ctypes.byref(params), _ptr(a), len(a))
        else:
            self.h = getattr(L, self.pre + "new_seed")(ctypes.byref(params), seed)
        self.size = getattr(L, self.pre + "size")(self.h)
        self.lsize = 1
        while self.lsize <= self.size:
            self.lsize <<= 1

    def __del__(self):
        try:
            getattr(self.o.L, self.pre + "delete")(self.h)
        except Exception:
            pass

    def clone(self):
        h = getattr(self.o.L, self.pre + "clone")(self.h)
        return OracleGen(self.o, self.params, _h=h)

    def fill(self, kind, n):
        if self.bits == 32:
            dt = np.uint32 if kind == 0 else np.float32
        else:
            dt = np.uint64 if kind == 0 else np.float64
        out = np.empty(n, dtype=dt)
        getattr(self.o.L, self.pre + "fill")(self.h, kind, _ptr(out), n)
        return out

    def skip(self, n):
        getattr(self.o.L, self.pre + "skip")(self.h, n)

    def fast_jump(self, hexstr):
        rc = getattr(self.o.L, self.pre + "fast_jump")(self.h, hexstr.encode())
        if rc:
            raise ValueError("bad jump string")

    def jump_words(self, words):
        w = np.ascontiguousarray(words, np.uint32)
        getattr(self.o.L, self.pre + "jump_words")(self.h, _ptr(w), len(w))

    def window(self):
        out = np.empty(self.size, dtype=self.wdt)
        getattr(self.o.L, self.pre + "get_window")(self.h, _ptr(out))
        return out

    def set_window(self, win):
        w = np.ascontiguousarray(win, self.wdt)
        getattr(self.o.L, self.pre + "set_window")(self.h, _ptr(w))

    def ring(self):
        out = np.empty(self.lsize, dtype=self.wdt)
        idx = getattr(self.o.L, self.pre + "get_ring")(self.h, _ptr(out))
        return idx, out


class Reference:
    """The reference library itself (oracle/_ref), where it was built."""

    def __init__(self):
        if not os.path.exists(REFLIB):
            raise FileNotFoundError(REFLIB)
        L = ctypes.CDLL(REFLIB)
        self.L = L
        L.ref_table.restype = _P
        L.ref_table.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
        for s in ("ref_jump_string32", "ref_jump_string64", "ref_char32_11213"):
            getattr(L, s).restype = ctypes.c_char_p
        for b, pt in ((32, MTGP32Params), (64, MTGP64Params)):
            wt = ctypes.c_uint32 if b == 32 else ctypes.c_uint64
            pre = "ref%d_" % b
            getattr(L, pre + "new").restype = _P
            getattr(L, pre + "new").argtypes = [ctypes.POINTER(pt), ctypes.c_int, wt, _P,
                                                ctypes.c_int, ctypes.c_char_p]
            getattr(L, pre + "delete").argtypes = [_P]
            getattr(L, pre + "fill").argtypes = [_P, ctypes.c_int, _P, ctypes.c_size_t]
            getattr(L, pre + "fast_jump").argtypes = [_P, ctypes.c_char_p]
            getattr(L, pre + "ring").argtypes = [_P, _P]
            getattr(L, pre + "multi_seed_fill").argtypes = [
                ctypes.POINTER(pt), _P, _P, ctypes.c_int, _P, _P, _P, _P, ctypes.c_int]
        L.ref32_print_idstring.argtypes = [_P, ctypes.c_char_p, ctypes.c_int]

    def table_raw(self, name, cls):
        n = ctypes.c_int()
        p = self.L.ref_table(name.encode(), ctypes.byref(n))
        return (cls * n.value).from_address(p), n.value

    def max_threads(self):
        return self.L.ref_max_threads()

    def gen(self, params, seed=None, array=None, string=None):
        return RefGen(self, params, seed, array, string)


class RefGen:
    def __init__(self, ref, params, seed=None, array=None, string=None):
        self.r = ref
        self.bits = 32 if isinstance(params, MTGP32Params) else 64
        self.pre = "ref%d_" % self.bits
        self.wdt = np.uint32 if self.bits == 32 else np.uint64
        f = getattr(ref.L, self.pre + "new")
        if string is not None:
            self._s = ctypes.create_string_buffer(string)
            self.h = f(ctypes.byref(params), 2, 0, None, 0, self._s)
        elif array is not None:
            self._a = np.ascontiguousarray(array, self.wdt)
            self.h = f(ctypes.byref(params), 1, 0, _ptr(self._a), len(self._a), None)
        else:
            self.h = f(ctypes.byref(params), 0, seed, None, 0, None)
        self.size = params.mexp // self.bits + 1
        self.lsize = 1
        while self.lsize <= self.size:
            self.lsize <<= 1

    def __del__(self):
        try:
            getattr(self.r.L, self.pre + "delete")(self.h)
        except Exception:
            pass

    def fill(self, kind, n):
        if self.bits == 32:
            dt = np.uint32 if kind == 0 else np.float32
        else:
            dt = np.uint64 if kind == 0 else np.float64
        out = np.empty(n, dtype=dt)
        getattr(self.r.L, self.pre + "fill")(self.h, kind, _ptr(out), n)
        return out

    def fast_jump(self, hexstr):
        getattr(self.r.L, self.pre + "fast_jump")(self.h, hexstr.encode())

    def ring(self):
        out = np.empty(self.lsize, dtype=self.wdt)
        idx = getattr(self.r.L, self.pre + "ring")(self.h, _ptr(out))
        return idx, out

    def window(self):
        idx, ring = self.ring()
        return np.array([ring[(idx - self.size + 1 + k) % self.lsize]
                         for k in range(self.size)], dtype=self.wdt)
