"""GF(2) jump-ahead on the GPU vs the oracle (mtgp32-fast-jump.c:51-79)."""
import numpy as np
import pytest
import torch

from mtgp_gb300.params import jump_string, jump_table, load_table

pytestmark = pytest.mark.gpu


def same_state(g, o, p):
    """States agree: word 0 under the state mask (its other bits never reach
    an output, mtgp32-fast.h:149-159; the reference compares it the same way,
    cuda-sample/mtgp32-sample-jump1-host.cu:105-108), every other word
    exactly, and the next outputs exactly."""
    a, b = g.window(), o.clone().window()
    if (int(a[0]) ^ int(b[0])) & int(p.mask):
        return False
    if not np.array_equal(a[1:], b[1:]):
        return False
    nxt = g.fill(0, 2000).cpu().numpy().view(a.dtype)
    return np.array_equal(nxt, o.clone().fill(0, 2000))

CASES = [(32, "mtgp32_fast_11213"), (64, "mtgp64dc_fast_11213")]


def _gen(bits, p, **kw):
    from mtgp_gb300.api import MTGP32, MTGP64
    return (MTGP32 if bits == 32 else MTGP64)(p, **kw)


@pytest.mark.parametrize("bits,table", CASES)
def test_fast_jump_string(gpu, orc, bits, table):
    p = load_table(table)[0]
    g = _gen(bits, p, seed=1234)
    o = orc.gen(p, seed=1234)
    g.fill(0, 777)
    o.fill(0, 777)
    g.fast_jump(jump_string(bits))
    o.fast_jump(jump_string(bits))
    assert np.array_equal(g.window(), o.window())
    assert np.array_equal(g.fill(0, 4000).cpu().numpy().view(o.window().dtype), o.fill(0, 4000))


@pytest.mark.parametrize("bits,table", CASES)
def test_jump_table_rows(gpu, orc, bits, table):
    p = load_table(table)[0]
    tbl = jump_table(bits)
    g = _gen(bits, p, seed=1)
    o = orc.gen(p, seed=1)
    for row in (5, 1, 3):
        g.jump_array(tbl[row])
        o.jump_words(tbl[row])
        assert np.array_equal(g.window(), o.window()), row


@pytest.mark.parametrize("bits,table,idx", [(32, "mtgp32_fast_23209", 2), (32, "mtgp32_fast_44497", 1),
                                            (64, "mtgp64_fast_23209", 0), (64, "mtgp64_fast_44497", 3),
                                            (64, "mtgp64_fast_110503", 0)])
def test_jump_other_exponents(gpu, orc, bits, table, idx):
    """Random polynomials on every exponent's kernel shape (output groups,
    ring sizes, wide lanes)."""
    p = load_table(table)[idx]
    rng = np.random.default_rng(idx + bits)
    nwords = p.mexp // 32 + 1
    poly = rng.integers(0, 2 ** 32, nwords, dtype=np.uint64).astype(np.uint32)
    poly[-1] &= (1 << (p.mexp % 32)) - 1
    g = _gen(bits, p, seed=11)
    o = orc.gen(p, seed=11)
    g.jump_array(poly)
    o.jump_words(poly)
    assert np.array_equal(g.window(), o.window())


def test_jump_small_polys(gpu, orc):
    """Polynomials X^k for small k: jump == k steps (test-jump32.cpp:224-229)."""
    for bits, table in CASES:
        p = load_table(table)[0]
        for k in (0, 1, 2, 31, 32, 33, 351, 1000):
            poly = np.zeros(k // 32 + 1, dtype=np.uint32)
            poly[k // 32] = 1 << (k % 32)
            g = _gen(bits, p, seed=3)
            o = orc.gen(p, seed=3)
            g.jump_array(poly)
            o.skip(k)
            assert np.array_equal(g.window(), o.window()), (bits, k)


@pytest.mark.parametrize("bits,table", CASES + [(32, "mtgp32_fast_44497"),
                                                (64, "mtgp64_fast_110503")])
def test_jump_steps_equals_skip(gpu, orc, bits, table):
    """jump_steps makes X^s mod chi on the GPU (chi by Berlekamp-Massey over
    GPU output, then products from the byte-window tables; the 2-bit-window
    product kernel for the longest exponent) and jumps on the GPU."""
    p = load_table(table)[0]
    for steps in (1, 1000, 123457, (1 << 22) + 3):
        g = _gen(bits, p, seed=8)
        o = orc.gen(p, seed=8)
        g.jump_steps(steps)
        o.skip(steps)
        assert same_state(g, o, p), steps


def test_jump_steps_large_exponent(gpu, orc):
    """A 127-bit step count: X^s mod chi from the host GF(2) code (the
    GPU schedules take 64-bit distances) equals the oracle's bit-serial
    PowerXMod, so the windows agree exactly."""
    p = load_table("mtgp32_fast_11213")[0]
    steps = 3 ** 80
    assert steps < 2 ** 128
    bits_seq = (orc.gen(p, seed=1).fill(0, 2 * p.mexp) & 1).astype(np.uint8)
    d, chi = orc.minpoly(bits_seq)
    poly = orc.powxmod(steps, chi, d).view(np.uint32)[:351]
    g = _gen(32, p, seed=1234)
    o = orc.gen(p, seed=1234)
    g.jump_steps(steps)
    o.jump_words(poly)
    assert np.array_equal(g.window(), o.window())


def test_jump_steps_rejects_oversized(gpu):
    g = _gen(32, load_table("mtgp32_fast_11213")[0], seed=1)
    with pytest.raises(ValueError):
        g.jump_steps(2 ** 128)


@pytest.mark.parametrize("bits,table", CASES)
def test_substreams(gpu, orc, bits, table):
    """Substream j = seed state jumped by j * 3^162 on the GPU.  Exact against
    the oracle walking the same table rows (bit b of j applies row b/2 once
    for even b, twice for odd b: cuda-sample/mtgp32-jump-kernel.cuh:383-401);
    equal as a state (word 0 under the mask, outputs exact) to j successive
    JUMP3_162 jumps of the reference's CPU code.  1000 substreams: the GPU
    makes them by doubling in ten levels, the last one partial."""
    from mtgp_gb300.api import Pool
    p = load_table(table)[0]
    tbl = jump_table(bits)
    count = 1000
    pool = Pool.substreams(p, 1234, count, tbl)
    win = pool.windows()
    chain = orc.gen(p, seed=1234)
    js = jump_string(bits)
    for j in list(range(70)) + [255, 256, 511, 512, 513, 767, 998, 999]:
        o = orc.gen(p, seed=1234)
        for b in range(12):
            if (j >> b) & 1:
                o.jump_words(tbl[b // 2])
                if b & 1:
                    o.jump_words(tbl[b // 2])
        assert np.array_equal(win[j], o.window()), j
        if j < 70:
            c = chain.clone()
            w = c.window()
            assert (int(w[0]) ^ int(win[j][0])) & int(p.mask) == 0, j
            assert np.array_equal(w[1:], win[j][1:]), j
            chain.fast_jump(js)


@pytest.mark.parametrize("bits,table,idx,window", [(32, "mtgp32_fast_11213", 0, 0),
                                                   (32, "mtgp32_fast_11213", 3, 2),
                                                   (64, "mtgp64dc_fast_11213", 1, 0),
                                                   (32, "mtgp32_fast_23209", 2, 0),
                                                   (32, "mtgp32_fast_44497", 1, 0)])
def test_gpu_jump_polys_match_oracle(gpu, orc, bits, table, idx, window):
    """X^e mod chi computed on the GPU (byte-window tables made on the GPU,
    then a tree of comb products with Barrett reduction) equals the oracle's
    bit-serial PowerXMod; window 2 is the variant for long polynomials."""
    from mtgp_gb300.api import Pool, set_tuning
    tbl = load_table(table)
    set_tuning("poly_window", window)
    try:
        pool = Pool.create([tbl[0], tbl[idx]], [1, 2], [0, 1])
        p = tbl[idx]
        rng = np.random.default_rng(31 + idx)
        steps = [0, 1, 2, 3, 255, 256, 1 << 17, (1 << 40) + 12345, (1 << 64) - 1, 3 ** 40]
        nrand = 2 if p.mexp > 40000 else 8
        steps += [int(x) for x in rng.integers(0, 2 ** 63, nrand, dtype=np.int64)]
        got = pool.jump_polys(1, steps).cpu().numpy().view(np.uint32)
    finally:
        set_tuning("poly_window", 0)
    seq = orc.gen(p, seed=1).fill(0, 2 * p.mexp)
    d, chi = orc.minpoly((seq & 1).astype(np.uint8))
    nw = p.mexp // 32 + 1
    for k, e in enumerate(steps):
        ref = orc.powxmod(e, chi, d).view(np.uint32)[:nw]
        assert np.array_equal(got[k], ref), e


def test_gpu_jump_polys_many(gpu, orc):
    """600 exponents at once (one chain of products per CTA instead of the
    tree): 40 distinct exponents, each repeated, against the oracle."""
    from mtgp_gb300.api import Pool
    tbl = load_table("mtgp32_fast_11213")
    p = tbl[5]
    pool = Pool.create([p], [3], [0])
    rng = np.random.default_rng(8)
    distinct = [int(x) for x in rng.integers(0, 2 ** 63, 40, dtype=np.int64)]
    steps = [distinct[(7 * k) % 40] for k in range(600)]
    got = pool.jump_polys(0, steps).cpu().numpy().view(np.uint32)
    seq = orc.gen(p, seed=1).fill(0, 2 * p.mexp)
    d, chi = orc.minpoly((seq & 1).astype(np.uint8))
    nw = p.mexp // 32 + 1
    refs = {e: orc.powxmod(e, chi, d).view(np.uint32)[:nw] for e in distinct}
    for k, e in enumerate(steps):
        assert np.array_equal(got[k], refs[e]), (k, e)
