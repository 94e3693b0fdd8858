"""The library's host GF(2)[x] arithmetic (table reduction, comb products,
X^e by squaring and by products of X^(2^i)) equals the oracle's bit-serial
PowerXMod / MulMod on the characteristic polynomials of the shipped
parameter sets (CPU only)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from mtgp_gb300.params import load_table

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("gf2") / "gf2_probe.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", so,
                    os.path.join(HERE, "gf2_probe.cpp"),
                    os.path.join(ROOT, "mtgp_gb300", "csrc", "gf2.cpp")], check=True)
    L = ctypes.CDLL(so)
    vp = ctypes.c_void_p
    L.probe_powx.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int, vp]
    L.probe_mulmod.argtypes = [vp, vp, vp, ctypes.c_int, vp]
    L.probe_pow2_product.argtypes = [vp, ctypes.c_int, ctypes.c_uint64, vp]
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _chi(orc, table):
    p = load_table(table)[0]
    seq = orc.gen(p, seed=1).fill(0, 2 * p.mexp)
    d, chi = orc.minpoly((seq & 1).astype(np.uint8))
    assert d == p.mexp
    m = np.zeros(d // 64 + 1, dtype=np.uint64)
    m[:min(len(chi), len(m))] = chi[:len(m)]
    return d, m


TABLES = ["mtgp32_fast_11213", "mtgp64dc_fast_11213", "mtgp32_fast_23209"]
EXPS = [1, 2, 63, 64, 65, 1 << 17, (1 << 40) + 12345, 3 ** 40, (1 << 64) - 1, 3 ** 80]


@pytest.mark.parametrize("table", TABLES)
def test_powx_matches_oracle(orc, probe, table):
    d, m = _chi(orc, table)
    for e in EXPS:
        ew = max(1, (e.bit_length() + 31) // 32)
        ea = np.array([(e >> (32 * k)) & 0xffffffff for k in range(ew)], dtype=np.uint32)
        out = np.zeros((d + 63) // 64, dtype=np.uint64)
        probe.probe_powx(_p(m), d, _p(ea), ew, _p(out))
        assert np.array_equal(out, orc.powxmod(e, m, d)), e
        if e < (1 << 64):
            out2 = np.zeros_like(out)
            probe.probe_pow2_product(_p(m), d, e, _p(out2))
            assert np.array_equal(out2, out), e


@pytest.mark.parametrize("table", TABLES[:2])
def test_mulmod_matches_oracle(orc, probe, table):
    d, m = _chi(orc, table)
    rng = np.random.default_rng(9)
    w = (d + 63) // 64
    top = np.uint64((1 << (d % 64)) - 1)
    for _ in range(4):
        a = rng.integers(0, 2 ** 63, w, dtype=np.uint64) * np.uint64(2) + np.uint64(1)
        b = rng.integers(0, 2 ** 63, w, dtype=np.uint64) * np.uint64(3)
        a[-1] &= top
        b[-1] &= top
        out = np.zeros(w, dtype=np.uint64)
        probe.probe_mulmod(_p(a), _p(b), _p(m), d, _p(out))
        assert np.array_equal(out, orc.mulmod(a, b, m, d))


def test_barrett_constant(orc, probe):
    """mu = floor(X^(2d) / chi) satisfies X^(2d) = mu * chi + rho with
    deg rho < d (checked with the oracle's products)."""
    probe.probe_divxpow.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    d, m = _chi(orc, "mtgp32_fast_11213")
    mu = np.zeros(d // 64 + 2, dtype=np.uint64)
    n = probe.probe_divxpow(_p(m), d, 2 * d, _p(mu))
    assert n == d // 64 + 1
    # the bit-serial product mu * chi, then X^(2d) xor it must have degree < d
    prod = np.zeros(2 * d // 64 + 3, dtype=np.uint64)
    for i in range(d + 1):
        if (int(mu[i >> 6]) >> (i & 63)) & 1:
            for k in range(len(m)):
                w = int(m[k])
                if not w:
                    continue
                lo = (w << (i & 63)) & (2 ** 64 - 1)
                hi = w >> (64 - (i & 63)) if i & 63 else 0
                prod[k + (i >> 6)] ^= np.uint64(lo)
                if hi:
                    prod[k + (i >> 6) + 1] ^= np.uint64(hi)
    prod[(2 * d) >> 6] ^= np.uint64(1 << ((2 * d) & 63))
    top = max((64 * k + int(prod[k]).bit_length() - 1 for k in range(len(prod)) if prod[k]),
              default=-1)
    assert top < d


def test_pow_schedules_match_oracle(orc, probe):
    """The GPU's product schedules (byte-window table, then per exponent a
    serial chain or a pairwise tree), executed here with the host's
    products, give the oracle's X^e mod chi; the tree is picked for few
    exponents (depth 3 for eight factors), the chain for many."""
    L = probe
    vp = ctypes.c_void_p
    L.probe_pow_schedule.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int, vp, vp]
    d, m = _chi(orc, "mtgp32_fast_11213")
    w = (d + 63) // 64
    rng = np.random.default_rng(5)
    exps = np.array([0, 1, 255, 256, 257, (1 << 64) - 1, 1 << 63, 0x0101010101010101,
                     *rng.integers(0, 2 ** 63, 6, dtype=np.uint64)], dtype=np.uint64)
    for width, want in ((152, "tree"), (1, "serial")):
        out = np.zeros((len(exps), w), dtype=np.uint64)
        shape = np.zeros(3, dtype=np.int32)
        assert L.probe_pow_schedule(_p(m), d, _p(exps), len(exps), width, _p(out), _p(shape)) == 0
        for j, e in enumerate(exps):
            assert np.array_equal(out[j], orc.powxmod(int(e), m, d)), (width, int(e))
        levels, steps, nscratch = shape
        if want == "tree":
            assert levels == 3 and nscratch > 0
        else:
            assert levels == 1 and steps == len(exps) and nscratch == 0


@pytest.mark.parametrize("table", ["mtgp32_fast_11213", "mtgp64dc_fast_11213"])
def test_gpu_formulations_of_bm_and_barrett(orc, probe, table):
    """The formulations of the GPU's Berlekamp-Massey (bit-reversed sequence,
    discrepancy as the parity of a shifted window) and Barrett constant
    (power-series inverse of chi's reciprocal), restated serially: the
    oracle's characteristic polynomial, and the host's floor(X^(2d)/chi)."""
    vp = ctypes.c_void_p
    probe.probe_bm_reversed.argtypes = [vp, ctypes.c_int, vp]
    probe.probe_barrett_series.argtypes = [vp, ctypes.c_int, vp]
    probe.probe_divxpow.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp]
    p = load_table(table)[2]
    seq = (orc.gen(p, seed=1).fill(0, 2 * p.mexp) & 1).astype(np.uint8)
    d, chi = orc.minpoly(seq)
    out = np.zeros(len(chi) + 2, dtype=np.uint64)
    assert probe.probe_bm_reversed(_p(seq), len(seq), _p(out)) == d
    assert np.array_equal(out[:d // 64 + 1], chi[:d // 64 + 1])
    m = np.ascontiguousarray(chi[:d // 64 + 1])
    mu = np.zeros(d // 64 + 2, dtype=np.uint64)
    probe.probe_barrett_series(_p(m), d, _p(mu))
    ref = np.zeros(d // 64 + 2, dtype=np.uint64)
    nq = probe.probe_divxpow(_p(m), d, 2 * d, _p(ref))
    assert np.array_equal(mu[:nq], ref[:nq]) and not mu[nq:].any()
