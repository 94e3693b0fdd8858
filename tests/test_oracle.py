"""The oracle (CPU restatement of the reference) pinned against the
reference's own outputs: golden vectors made by the reference compiled from
its sources (tests/golden/make_golden.py), the reference library itself when
it is built here (oracle/_ref), and the shipped polynomials."""
import os

import numpy as np
import pytest

from mtgp_gb300.params import (characteristic_string, jump_string, jump_table,
                               load_table)

from golden.make_golden import CASES, HIGH_KEY  # noqa: E402

REFLIB = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                      "oracle", "_ref", "libmtgpref.so")


@pytest.mark.parametrize("table,idx,n", CASES)
def test_oracle_matches_golden(orc, golden, table, idx, n):
    p = load_table(table)[idx]
    key = "%s_%d" % (table, idx)
    assert np.array_equal(orc.gen(p, seed=1).fill(0, n), golden[key + "_seed1_uint"])
    assert np.array_equal(orc.gen(p, array=[1, 2, 3, 4]).fill(0, n), golden[key + "_array1234_uint"])
    g = orc.gen(p, string=b"\x01\x02\x03\x04")
    assert np.array_equal(g.fill(0, n), golden[key + "_str1234_uint"])
    for kind in (1, 2, 3, 4):
        got = g.fill(kind, n)
        assert got.tobytes() == golden[key + "_str1234_kind%d" % kind].tobytes(), kind
    assert np.array_equal(orc.gen(p, string=HIGH_KEY).fill(0, n), golden[key + "_highkey_uint"])


@pytest.mark.parametrize("bits,table", [(32, "mtgp32_fast_11213"), (64, "mtgp64dc_fast_11213")])
def test_oracle_jump_matches_golden(orc, golden, bits, table):
    p = load_table(table)[0]
    g = orc.gen(p, seed=1234)
    g.fill(0, 777)
    g.fast_jump(jump_string(bits))
    idx, ring = g.ring()
    assert idx == golden["jump%d_idx" % bits][0]
    assert np.array_equal(ring, golden["jump%d_ring" % bits])
    assert np.array_equal(g.fill(0, 512), golden["jump%d_next_uint" % bits])


@pytest.mark.parametrize("bits,table", [(32, "mtgp32_fast_11213"), (64, "mtgp64dc_fast_11213")])
def test_oracle_characteristic_and_jump_polynomials(orc, bits, table):
    """Berlekamp-Massey over 2*mexp output LSBs (mtgp32-calc-poly.cpp:36-45)
    reproduces the shipped characteristic polynomial, and X^(3^162) mod chi
    reproduces the shipped jump string and jump-table row 0."""
    p = load_table(table)[0]
    bits_seq = (orc.gen(p, seed=1).fill(0, 2 * p.mexp) & 1).astype(np.uint8)
    d, chi = orc.minpoly(bits_seq)
    assert d == p.mexp
    assert orc.to_hex(chi, d) == characteristic_string(bits)
    jp = orc.powxmod(3 ** 162, chi, d)
    deg = max(i for i in range(d) if (int(jp[i // 64]) >> (i % 64)) & 1)
    assert orc.to_hex(jp, deg) == jump_string(bits)
    assert np.array_equal(jump_table(bits)[0], jp.view(np.uint32)[:351])


def test_oracle_jump_equals_stepping(orc):
    """A jump by X^s mod chi equals s plain steps (test-jump32.cpp:154-173)."""
    p = load_table("mtgp32_fast_11213")[0]
    bits_seq = (orc.gen(p, seed=1).fill(0, 2 * p.mexp) & 1).astype(np.uint8)
    d, chi = orc.minpoly(bits_seq)
    for steps in (1, 2, 352, 32 * 351 + 1, 3003):
        a = orc.gen(p, seed=4321)
        b = a.clone()
        a.skip(steps)
        jp = orc.powxmod(steps, chi, d)
        b.jump_words(jp.view(np.uint32)[:351])
        assert np.array_equal(a.fill(0, 100), b.fill(0, 100)), steps


def test_oracle_bad_jump_string(orc):
    g = orc.gen(load_table("mtgp32_fast_11213")[0], seed=1)
    with pytest.raises(ValueError):
        g.fast_jump("12x4")


def test_oracle_multi_fill_matches_single(orc):
    tbl = load_table("mtgp32_fast_11213")
    from mtgp_gb300.params import params_array, MTGP32Params
    params = params_array(MTGP32Params, [tbl[i] for i in range(8)])
    seeds = np.arange(8, dtype=np.uint32) + 1234
    win = orc.seed_windows(32, params, seeds)
    counts = np.array([0, 1, 255, 1000, 7, 4096, 33, 512], dtype=np.uint64)
    offs = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint64) * 4
    out = np.zeros(int(counts.sum()), dtype=np.uint32)
    orc.multi_fill(32, params, win, counts, np.zeros(8, np.int32), offs, out)
    for i in range(8):
        ref = orc.gen(tbl[i], seed=int(seeds[i])).fill(0, int(counts[i]))
        o = int(offs[i]) // 4
        assert np.array_equal(out[o:o + int(counts[i])], ref)


@pytest.mark.skipif(not os.path.exists(REFLIB), reason="reference library not built here")
def test_oracle_matches_reference_library(orc):
    """Direct comparison with the reference compiled from its own sources."""
    from oracle.bind import Reference
    ref = Reference()
    for table, idxs in (("mtgp32_fast_11213", (0, 64, 127)), ("mtgp32dc_fast_11213", (0, 199)),
                        ("mtgp32_fast_44497", (3,)), ("mtgp64dc_fast_11213", (0, 100)),
                        ("mtgp64_fast_110503", (5,))):
        for idx in idxs:
            p = load_table(table)[idx]
            for kw in (dict(seed=99), dict(array=[7, 8, 9]), dict(string=b"\xfe\x01xyz")):
                a, b = orc.gen(p, **kw), ref.gen(p, **kw)
                for kind in range(5):
                    assert a.fill(kind, 2000).tobytes() == b.fill(kind, 2000).tobytes()
