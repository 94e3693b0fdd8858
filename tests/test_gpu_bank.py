"""Generator banks (one CTA per parameter set): configs 2 and 3 at reduced
length and at full length, bit-exact per stream."""
import numpy as np
import pytest
import torch

from mtgp_gb300.params import load_table
from gpu_util import as_np_bits, np_bits

pytestmark = pytest.mark.gpu


def _bank(orc, bits, table, base_seed, count, n, kinds):
    from mtgp_gb300.api import Pool
    from mtgp_gb300.params import params_array, MTGP32Params, MTGP64Params
    tbl = load_table(table)
    plist = [tbl[i] for i in range(count)]
    seeds = np.arange(count) + base_seed
    pool = Pool.create(plist, seeds)
    P = MTGP32Params if bits == 32 else MTGP64Params
    parr = params_array(P, plist)
    win = orc.seed_windows(bits, parr, seeds)
    for kind in kinds:
        dt = {32: (torch.int32, torch.float32), 64: (torch.int64, torch.float64)}[bits][kind != 0]
        out = torch.empty(count * n, dtype=dt, device="cuda")
        pool.fill(kind, out, n)
        torch.cuda.synchronize()
        got = as_np_bits(out, bits)
        ref = np.zeros(count * n, dtype=np.uint32 if bits == 32 else np.float32)
        ref = np.zeros(count * n, dtype={32: (np.uint32, np.float32), 64: (np.uint64, np.float64)}[bits][kind != 0])
        esz = bits // 8
        orc.multi_fill(bits, parr, win, np.full(count, n, np.uint64), np.full(count, kind, np.int32),
                       np.arange(count, dtype=np.uint64) * n * esz, ref)
        assert np.array_equal(got, np_bits(ref, bits)), kind
    assert np.array_equal(pool.windows(), win)


def test_config2_bank_reduced(gpu, orc):
    _bank(orc, 32, "mtgp32_fast_11213", 1234, 128, 1 << 14, (0, 2))


def test_config3_bank_reduced(gpu, orc):
    _bank(orc, 64, "mtgp64dc_fast_11213", 5678, 200, 1 << 13, (0, 1))


def test_config2_bank_full_length(gpu, orc):
    """128 sets x 2^21 uint32, then 2^21 float [0,1) each: full size."""
    _bank(orc, 32, "mtgp32_fast_11213", 1234, 128, 1 << 21, (0, 2))


def test_config3_bank_full_length(gpu, orc):
    """200 sets of the OpenCL mtgp64dc table x 2^20 uint64, then 2^20 double
    [1,2) each (mantissa bit-packing): full size."""
    _bank(orc, 64, "mtgp64dc_fast_11213", 5678, 200, 1 << 20, (0, 1))


def test_other_mexp_banks(gpu, orc):
    _bank(orc, 32, "mtgp32_fast_44497", 1, 16, 5000, (0, 4))
    _bank(orc, 64, "mtgp64_fast_110503", 1, 16, 3000, (0, 3))
