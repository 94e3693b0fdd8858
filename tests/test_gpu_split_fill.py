"""Large fills of a single generator run split across many CTAs (chunks
start from windows jumped by X^(c * chunk), made by jump parts before the
chunks run, or inside the kernel): the values, the sequence continued by
later fills and the exported state equal the reference loop's, for
back-to-back fills issued without synchronisation."""
import numpy as np
import pytest
import torch

from mtgp_gb300.params import load_table
from gpu_util import check_guards, guarded, np_bits

pytestmark = pytest.mark.gpu

CASES = [(32, "mtgp32_fast_11213", 0), (64, "mtgp64dc_fast_11213", 0),
         (32, "mtgp32_fast_23209", 1), (64, "mtgp64_fast_23209", 2)]


# (jump_parts, single_chunk): automatic; three CTAs per jump with an odd
# chunk length; one CTA per jump; chunks that jump inside the batched kernel
TUNINGS = [(0, 0), (3, 100003), (1, 0), (-1, 0)]


@pytest.fixture
def tuning(request):
    from mtgp_gb300.api import set_tuning
    parts, chunk = request.param
    set_tuning("jump_parts", parts)
    set_tuning("single_chunk", chunk)
    yield request.param
    set_tuning("jump_parts", 0)
    set_tuning("single_chunk", 0)


@pytest.mark.parametrize("tuning", TUNINGS, indirect=True)
@pytest.mark.parametrize("bits,table,idx", CASES)
def test_split_fills_continue_the_sequence(gpu, orc, bits, table, idx, tuning):
    from mtgp_gb300.api import MTGP32, MTGP64
    p = load_table(table)[idx]
    g = (MTGP32 if bits == 32 else MTGP64)(p, seed=4321)
    o = orc.gen(p, seed=4321)
    s = torch.cuda.Stream()
    plan = [(0, (1 << 20) + 7), (2, 3 << 20), (1, 1000), (4, (1 << 21) + 1), (3, 1 << 20), (0, 5)]
    outs = []
    for kind, n in plan:                 # issued back to back on one stream
        full, view = guarded(n, bits, kind)
        g.fill_into(kind, view, n, stream=s)
        outs.append(full)
    s.synchronize()
    for (kind, n), full in zip(plan, outs):
        check_guards(full, bits)
        got = np_bits(full[64:64 + n].cpu().numpy(), bits)
        assert np.array_equal(got, np_bits(o.fill(kind, n), bits)), (kind, n)
    assert np.array_equal(g.window(), o.window())
