"""First use of many parameter sets in one plan: their characteristic
polynomials (Berlekamp-Massey on the GPU), Barrett constants, X^(2^i) chains
and jump tables are made in one batch, and the chunk offsets of split
requests are computed together on the GPU.  Outputs against the oracle."""
import numpy as np
import pytest
import torch

from mtgp_gb300.params import load_table
from gpu_util import as_np_bits

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bits,table,nsets", [(32, "mtgp32_fast_11213", 24),
                                              (64, "mtgp64dc_fast_11213", 12)])
def test_many_sets_split_requests(gpu, orc, bits, table, nsets):
    from mtgp_gb300.api import Pool, work_items
    tbl = load_table(table)
    plist = [tbl[i] for i in range(nsets)]
    seeds = np.arange(nsets) + 77
    pool = Pool.create(plist, seeds)
    n = (1 << 20) + 12345 if bits == 32 else (1 << 19) + 999
    esz = bits // 8
    pool.set_tuning("split_chunk", 1 << 17)
    items = work_items(np.arange(nsets), np.zeros(nsets), np.full(nsets, n),
                       np.arange(nsets) * n * esz)
    plan = pool.plan(items)
    desc = plan.describe()
    out = torch.zeros(nsets * n * esz // 4, dtype=torch.int32, device="cuda")
    plan.launch(out)
    torch.cuda.synchronize()
    assert desc["tasks"] > nsets and (desc["jumps"] or desc["prejumps"])
    got = as_np_bits(out.view(torch.int32 if bits == 32 else torch.int64), bits).reshape(nsets, n)
    for i in range(nsets):
        o = orc.gen(plist[i], seed=int(seeds[i]))
        assert np.array_equal(got[i], o.fill(0, n)), i
        assert np.array_equal(pool.windows()[i], o.window()), i


def test_jump_polys_of_many_sets(gpu, orc):
    """pool_jump_polys for the second of two sets after a 24-set plan made
    the tables: against the oracle's PowerXMod."""
    from mtgp_gb300.api import Pool
    tbl = load_table("mtgp32_fast_11213")
    p = tbl[17]
    pool = Pool.create([tbl[3], p], [1, 2])
    steps = [(1 << 40) + 3, 0x0123456789abcdef, 257]
    got = pool.jump_polys(1, steps).cpu().numpy().view(np.uint32)
    seq = orc.gen(p, seed=1).fill(0, 2 * p.mexp)
    d, chi = orc.minpoly((seq & 1).astype(np.uint8))
    for k, e in enumerate(steps):
        assert np.array_equal(got[k], orc.powxmod(e, chi, d).view(np.uint32)[:351]), e
