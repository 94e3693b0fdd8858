"""Skips inside batched work items (generated when short, GF(2) jump when
long), plan reuse, and the continuous-batching server: bit-exact vs the
oracle, the same result alone and in a mix, and admission under a device
memory budget."""
import numpy as np
import pytest
import torch

from mtgp_gb300.params import jump_table, load_table
from gpu_util import np_bits

pytestmark = pytest.mark.gpu

CASES = [(32, "mtgp32_fast_11213"), (64, "mtgp64dc_fast_11213")]
DT = {32: torch.int32, 64: torch.int64}


def _pool(bits, table, n, seed0=100):
    from mtgp_gb300.api import Pool
    tbl = load_table(table)
    plist = [tbl[i % 3] for i in range(3)]
    pidx = np.arange(n) % 3
    seeds = np.arange(n) + seed0
    return Pool.create(plist, seeds, pidx), plist, pidx, seeds


def _masked_equal(a, b, p):
    return ((int(a[0]) ^ int(b[0])) & int(p.mask)) == 0 and np.array_equal(a[1:], b[1:])


@pytest.mark.parametrize("bits,table", CASES)
def test_skip_items_vs_oracle(gpu, orc, bits, table):
    """Short skips are generated; skips of 2^17 or more (first item or
    later) start a new task that jumps inside the kernel; a jump followed by
    a long request that is split into chunks; an advance-only item."""
    from mtgp_gb300.api import work_items
    pool, plist, pidx, seeds = _pool(bits, table, 6)
    #        stream kind count    skip
    spec = [(0, 0, 1000, 100),
            (0, 2, 777, 5000),            # later item: generated skip
            (1, 0, 4000, 200000),         # first item: jump
            (1, 0, 100, 1 << 17),         # later item: a second task that jumps
            (2, 1, 3_000_000, (1 << 20) + 7),  # jump, then a split request
            (3, -1, 0, 300000),           # jump only
            (4, 3, 5000, 0),
            (5, 4, 2500, 131071)]         # just below the jump threshold
    esz = bits // 8
    offs, pos = [], 0
    for s, k, c, _ in spec:
        offs.append(pos)
        pos += c * esz if k >= 0 else 0
    items = work_items([x[0] for x in spec], [x[1] for x in spec], [x[2] for x in spec], offs,
                       [x[3] for x in spec])
    out = torch.zeros(pos // 4 + 16, dtype=torch.int32, device="cuda")
    pool.submit(items, out)
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint8)
    gens = {}
    for (s, k, c, sk), off in zip(spec, offs):
        o = gens.setdefault(s, orc.gen(plist[pidx[s]], seed=int(seeds[s])))
        o.skip(sk)
        if k < 0:
            o.skip(c)
            continue
        ref = np_bits(o.fill(k, c), bits).view(np.uint8)
        assert np.array_equal(got[off:off + ref.size], ref), (s, k, c, sk)
    w = pool.windows()
    for s, o in gens.items():
        assert _masked_equal(w[s], o.window(), plist[pidx[s]]), s


def test_skip_2_40_by_jump(gpu, orc):
    """A skip of 2^40 (far beyond stepping) equals the oracle's jump by
    X^(2^40) mod chi."""
    from mtgp_gb300.api import work_items
    pool, plist, pidx, seeds = _pool(32, "mtgp32_fast_11213", 3)
    steps = 1 << 40
    items = work_items([1], [0], [5000], [0], [steps])
    out = torch.zeros(5000, dtype=torch.int32, device="cuda")
    pool.submit(items, out)
    torch.cuda.synchronize()
    p = plist[pidx[1]]
    chi_bits = (orc.gen(p, seed=1).fill(0, 2 * p.mexp) & 1).astype(np.uint8)
    d, chi = orc.minpoly(chi_bits)
    poly = orc.powxmod(steps, chi, d).view(np.uint32)[:351]
    o = orc.gen(p, seed=int(seeds[1]))
    o.jump_words(poly)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), o.fill(0, 5000))


@pytest.mark.parametrize("bits,table", CASES)
def test_replan_reuses_plan(gpu, orc, bits, table):
    """One plan refilled with new items (more of them, so its buffers grow)
    keeps producing the oracle's sequence."""
    from mtgp_gb300.api import work_items
    pool, plist, pidx, seeds = _pool(bits, table, 12)
    gens = [orc.gen(plist[pidx[s]], seed=int(seeds[s])) for s in range(12)]
    rng = np.random.default_rng(5)
    plan = None
    for rnd, n in enumerate((3, 12, 7, 12)):
        streams = rng.permutation(12)[:n]
        counts = rng.integers(1, 30000, n)
        counts[0] = 2_500_000 if rnd == 1 else counts[0]   # one split request
        esz = bits // 8
        offs = np.concatenate([[0], np.cumsum(counts)[:-1]]) * esz
        items = work_items(streams, np.zeros(n), counts, offs)
        plan = pool.plan(items) if plan is None else pool.replan(items, plan)
        out = torch.zeros(int(counts.sum()), dtype=DT[bits], device="cuda")
        plan.launch(out)
        torch.cuda.synchronize()
        got = np_bits(out.cpu().numpy(), bits)
        for j in range(n):
            ref = gens[streams[j]].fill(0, int(counts[j]))
            o = int(offs[j]) // esz
            assert np.array_equal(got[o:o + counts[j]], ref), (rnd, j)


def _server_pools():
    from mtgp_gb300.api import Pool
    p32 = load_table("mtgp32_fast_11213")[0]
    p64 = load_table("mtgp64dc_fast_11213")[0]
    a = Pool.substreams(p32, 4321, 32, jump_table(32))
    b = Pool.substreams(p64, 4321, 8, jump_table(64))
    return a, b, p32, p64


def _oracle_streams(orc, pool, params):
    gens = []
    for row in pool.windows():
        o = orc.gen(params, seed=1)
        o.set_window(row)
        gens.append(o)
    return gens


def _trace(rng, n, nst32, nst64):
    reqs = []
    for _ in range(n):
        pool = int(rng.random() < 0.3)
        st = int(rng.integers(0, nst64 if pool else nst32))
        kind = int(rng.choice([0, 0, 0, 2, 1, 3, 4, -1]))
        count = int(min(rng.lognormal(np.log(20000), 1.5), 3_000_000))
        skip = 0
        u = rng.random()
        if u < 0.1:
            skip = 1 << int(rng.integers(17, 41))
        elif u < 0.2:
            skip = int(rng.integers(1, 5000))
        reqs.append((pool, st, kind, count, skip))
    return reqs


@pytest.mark.parametrize("retune", [False, True], ids=["quiet", "retuned"])
def test_server_vs_oracle(gpu, orc, retune):
    """A random trace through the server (several batches in flight, both
    pools, skips, advance-only requests) equals each stream's sequence
    replayed in submission order.  "retuned": meanwhile another thread keeps
    changing the process-wide tuning defaults and the knobs of an unrelated
    pool, which must not touch the server's plans."""
    import threading
    from mtgp_gb300.api import Pool, Server, set_tuning
    a, b, p32, p64 = _server_pools()
    ga, gb = _oracle_streams(orc, a, p32), _oracle_streams(orc, b, p64)
    # the oracle's jump polynomials for the jumped skips
    chis = {}
    for bits, p in ((32, p32), (64, p64)):
        seq = orc.gen(p, seed=1).fill(0, 2 * p.mexp)
        chis[bits] = orc.minpoly((seq & 1).astype(np.uint8))
    rng = np.random.default_rng(11)
    trace = _trace(rng, 300, 32, 8)
    srv = Server(a, b, budget_bytes=64 << 20, slots=3, max_batch=64)
    stop = threading.Event()

    def churn():
        other = Pool.create([p32], [5], [0])
        knobs = [("core", (1, 4, 2)), ("split_chunk", (-1, 1500, 0)),
                 ("batch_grid", (7, 0)), ("jump_parts", (-1, 3, 0))]
        k = 0
        while not stop.is_set():
            key, vals = knobs[k % len(knobs)]
            set_tuning(key, vals[(k // len(knobs)) % len(vals)])
            other.set_tuning(key, vals[(k // len(knobs) + 1) % len(vals)])
            k += 1
        for key, vals in knobs:
            set_tuning(key, vals[-1])

    th = threading.Thread(target=churn) if retune else None
    if th:
        th.start()
    try:
        outs, tickets = [], []
        for pool, st, kind, count, skip in trace:
            dst = None if kind < 0 else torch.empty(count, dtype=DT[32 if pool == 0 else 64],
                                                    device="cuda")
            outs.append(dst)
            tickets.append(srv.submit(pool, st, kind, count, dst, skip=skip))
        for t in tickets:
            assert srv.wait(t, 120.0) == 0
    finally:
        stop.set()
        if th:
            th.join()
    lat, status = srv.results()
    assert (status == 0).all() and (lat >= 0).all()
    done, nbytes, batches = srv.stats()
    assert done == len(trace) and batches >= 2
    srv.close()
    for (pool, st, kind, count, skip), dst in zip(trace, outs):
        bits = 32 if pool == 0 else 64
        o = (ga if pool == 0 else gb)[st]
        if skip >= (1 << 17):
            # skips up to 2^40: the oracle jumps by X^skip mod chi (outputs
            # equal stepping's)
            d, chi = chis[bits]
            o.jump_words(orc.powxmod(skip, chi, d).view(np.uint32)[:351])
        else:
            o.skip(skip)
        if kind < 0:
            o.skip(count)
            continue
        ref = o.fill(kind, count)
        assert np.array_equal(np_bits(dst.cpu().numpy(), bits), np_bits(ref, bits)), (pool, st)


def test_server_same_alone_and_in_mix(gpu):
    """Each stream's first request gives the same values when it is served
    alone and when it is batched with hundreds of others."""
    from mtgp_gb300.api import Server
    rng = np.random.default_rng(23)
    trace = _trace(rng, 400, 32, 8)
    a, b, _, _ = _server_pools()
    srv = Server(a, b, budget_bytes=256 << 20, slots=4, max_batch=512)
    outs = []
    for pool, st, kind, count, skip in trace:
        dst = torch.empty(max(count, 1), dtype=DT[32 if pool == 0 else 64], device="cuda")
        outs.append(dst)
        srv.submit(pool, st, max(kind, 0), count, dst, skip=skip)
    srv.drain()
    srv.close()
    seen = set()
    for j, (pool, st, kind, count, skip) in enumerate(trace):
        if (pool, st) in seen:
            continue
        seen.add((pool, st))
        a1, b1, _, _ = _server_pools()
        one = Server(a1, b1, budget_bytes=64 << 20, slots=1, max_batch=1)
        dst = torch.empty(max(count, 1), dtype=DT[32 if pool == 0 else 64], device="cuda")
        assert one.wait(one.submit(pool, st, max(kind, 0), count, dst, skip=skip)) == 0
        one.close()
        assert torch.equal(dst, outs[j]), (pool, st)
        if len(seen) >= 6:
            break


def test_server_budget_and_host_destination(gpu, orc):
    """Requests larger than the budget are refused; a queue whose total is
    many times the budget is admitted piece by piece; results land in pinned
    host memory."""
    from mtgp_gb300._lib import MTGPError
    from mtgp_gb300.api import Server
    a, b, p32, _ = _server_pools()
    ga = _oracle_streams(orc, a, p32)
    srv = Server(a, None, budget_bytes=1 << 20, slots=2, max_batch=8)
    with pytest.raises(MTGPError) as e:
        srv.submit(0, 0, 0, (1 << 18) + 1)
    assert e.value.code == -7
    with pytest.raises(MTGPError):
        srv.submit(1, 0, 0, 10)          # no 64-bit pool
    outs, tickets = [], []
    for k in range(40):
        dst = torch.empty(200_000, dtype=torch.int32).pin_memory()
        outs.append(dst)
        tickets.append(srv.submit(0, k % 32, 0, 200_000, dst))
    srv.drain()
    lat, st = srv.results()
    assert (st == 0).all()
    srv.close()
    for k in range(40):
        ref = ga[k % 32].fill(0, 200_000)
        assert np.array_equal(outs[k].numpy().view(np.uint32), ref), k


def test_server_zero_copy_result_and_budget_admission(gpu, orc):
    """A request without destination keeps its result in the device arena
    (zero-copy view); kept results count against the budget, so a request
    that does not fit waits until the space is released."""
    from mtgp_gb300._lib import MTGPError
    from mtgp_gb300.api import Server
    a, b, p32, _ = _server_pools()
    ga = _oracle_streams(orc, a, p32)
    srv = Server(a, b, budget_bytes=1 << 20, slots=2, max_batch=8)
    t1 = srv.submit(0, 3, 0, 100_000)
    assert srv.wait(t1) == 0
    v = srv.result(t1, torch.int32)
    assert v.numel() == 100_000
    assert np.array_equal(v.cpu().numpy().view(np.uint32), ga[3].fill(0, 100_000))
    t2 = srv.submit(0, 4, 2, 200_000)         # 800 KB: does not fit beside t1
    with pytest.raises(MTGPError) as e:
        srv.wait(t2, 0.5)
    assert e.value.code == -6
    srv.release(t1)
    assert srv.wait(t2, 30.0) == 0
    w = srv.result(t2, torch.float32)
    assert np.array_equal(w.cpu().numpy(), ga[4].fill(2, 200_000))
    srv.release(t2)
    with pytest.raises(MTGPError):
        srv.release(t2)
    srv.close()


def test_jumps_across_many_parameter_sets(gpu, orc):
    """Twenty parameter sets that all need in-kernel jumps (more than the
    pool keeps reduction tables for at once, so some are dropped and
    rebuilt): every split request and skip is still bit-exact."""
    from mtgp_gb300.api import Pool, work_items
    tbl = load_table("mtgp32_fast_11213")
    n = 20
    plist = [tbl[i] for i in range(n)]
    seeds = np.arange(n) + 900
    pool = Pool.create(plist, seeds, np.arange(n))
    counts = np.full(n, 5000)
    skips = np.where(np.arange(n) % 3 == 0, 1 << 17, 0)
    offs = np.arange(n) * 5000 * 4
    pool.set_tuning("split_chunk", 1200)
    for rep in range(2):
        out = torch.zeros(n * 5000, dtype=torch.int32, device="cuda")
        pool.submit(work_items(np.arange(n), np.zeros(n), counts, offs, skips), out)
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(np.uint32)
        for k in range(n):
            o = orc.gen(plist[k], seed=int(seeds[k]))
            o.skip(int(skips[k]) * (rep + 1) + 5000 * rep)
            assert np.array_equal(got[k * 5000:(k + 1) * 5000], o.fill(0, 5000)), (rep, k)


@pytest.mark.parametrize("bits,table", CASES)
def test_arbitrary_skips_use_gpu_polynomials(gpu, orc, bits, table):
    """Skips at arbitrary (not power-of-two) offsets: their jump polynomials
    are computed on the GPU at launch; outputs and windows match the oracle
    jumped by the same X^skip, over two launches of the plan."""
    from mtgp_gb300.api import work_items
    pool, plist, pidx, seeds = _pool(bits, table, 8)
    rng = np.random.default_rng(77 + bits)
    skips = [int(x) for x in rng.integers(1 << 17, 1 << 40, 8, dtype=np.int64)]
    skips[3] = 1 << 33                # a power of two: stays on the host
    skips[5] = (1 << 20) + 1          # two factors from one table
    counts = [1000 + 37 * k for k in range(8)]
    esz = bits // 8
    offs = list(np.concatenate([[0], np.cumsum(counts)[:-1]]) * esz)
    items = work_items(list(range(8)), [0] * 8, counts, offs, skips)
    plan = pool.plan(items)
    chis = {}
    gens = [orc.gen(plist[pidx[s]], seed=int(seeds[s])) for s in range(8)]
    nw = plist[0].mexp // 32 + 1
    for rep in range(2):
        out = torch.zeros(sum(counts) * esz // 4 + 4, dtype=torch.int32, device="cuda")
        plan.launch(out)
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(np.uint8)
        for s in range(8):
            p = plist[pidx[s]]
            if s % 3 not in chis:
                seq = orc.gen(p, seed=1).fill(0, 2 * p.mexp)
                chis[s % 3] = orc.minpoly((seq & 1).astype(np.uint8))
            d, chi = chis[s % 3]
            gens[s].jump_words(orc.powxmod(skips[s], chi, d).view(np.uint32)[:nw])
            ref = np_bits(gens[s].fill(0, counts[s]), bits).view(np.uint8)
            assert np.array_equal(got[offs[s]:offs[s] + ref.size], ref), (rep, s)


def test_gpu_polynomials_with_graph_and_refill(gpu, orc):
    """A plan whose run starts are made on the GPU, launched first through a
    CUDA graph (the products run before the capture, the replays reuse
    them), then refilled with other skips and launched plainly: every
    output matches the oracle."""
    from mtgp_gb300.api import work_items
    bits, table = 32, "mtgp32_fast_11213"
    pool, plist, pidx, seeds = _pool(bits, table, 6, seed0=300)
    gens = [orc.gen(plist[pidx[s]], seed=int(seeds[s])) for s in range(6)]
    chis = {}
    nw = plist[0].mexp // 32 + 1

    def check(skips, counts, out):
        offs = list(np.concatenate([[0], np.cumsum(counts)[:-1]]) * 4)
        got = out.cpu().numpy().view(np.uint8)
        for s in range(6):
            p = plist[pidx[s]]
            if s % 3 not in chis:
                seq = orc.gen(p, seed=1).fill(0, 2 * p.mexp)
                chis[s % 3] = orc.minpoly((seq & 1).astype(np.uint8))
            d, chi = chis[s % 3]
            gens[s].jump_words(orc.powxmod(skips[s], chi, d).view(np.uint32)[:nw])
            ref = gens[s].fill(0, counts[s]).view(np.uint8)
            assert np.array_equal(got[offs[s]:offs[s] + ref.size], ref), (skips[s], s)

    rng = np.random.default_rng(12)
    skips = [int(x) for x in rng.integers(1 << 17, 1 << 45, 6, dtype=np.int64)]
    counts = [777 + 100 * k for k in range(6)]
    offs = list(np.concatenate([[0], np.cumsum(counts)[:-1]]) * 4)
    plan = pool.plan(work_items(list(range(6)), [0] * 6, counts, offs, skips))
    out = torch.zeros(sum(counts) + 8, dtype=torch.int32, device="cuda")
    s = torch.cuda.Stream()
    for rep in range(2):
        plan.graph_launch(out, s)
        s.synchronize()
        check(skips, counts, out)
    skips2 = [int(x) for x in rng.integers(1 << 17, 1 << 45, 6, dtype=np.int64)]
    pool.replan(work_items(list(range(6)), [0] * 6, counts, offs, skips2), plan)
    plan.launch(out, s)
    s.synchronize()
    check(skips2, counts, out)


def test_huge_arbitrary_skips(gpu, orc):
    """Skips near 2^63 with every byte set (eight table factors, the full
    product tree) in a batched plan and on a single generator, against the
    oracle jumped by the same distances."""
    from mtgp_gb300.api import MTGP32, work_items
    p = load_table("mtgp32_fast_11213")[0]
    seq = orc.gen(p, seed=1).fill(0, 2 * p.mexp)
    d, chi = orc.minpoly((seq & 1).astype(np.uint8))
    nw = p.mexp // 32 + 1
    skips = [0x7edcba9876543211, (1 << 63) + 0x0101010101010101]
    # batched: two streams of one pool
    pool, plist, pidx, seeds = _pool(32, "mtgp32_fast_11213", 2, seed0=900)
    counts, offs = [3000, 2000], [0, 3000 * 4]
    plan = pool.plan(work_items([0, 1], [0, 0], counts, offs, skips))
    out = torch.zeros(5000 + 8, dtype=torch.int32, device="cuda")
    plan.launch(out)
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint32)
    for s in range(2):
        q = plist[pidx[s]]
        sq = orc.gen(q, seed=1).fill(0, 2 * q.mexp)
        dq, cq = orc.minpoly((sq & 1).astype(np.uint8))
        o = orc.gen(q, seed=int(seeds[s]))
        o.jump_words(orc.powxmod(skips[s], cq, dq).view(np.uint32)[:nw])
        ref = o.fill(0, counts[s])
        assert np.array_equal(got[offs[s] // 4:offs[s] // 4 + counts[s]], ref), s
    # single generator: skip() by the same distance
    g, o = MTGP32(p, seed=4321), orc.gen(p, seed=4321)
    g.skip(skips[0])
    o.jump_words(orc.powxmod(skips[0], chi, d).view(np.uint32)[:nw])
    assert np.array_equal(g.fill_uint32(2000).cpu().numpy().view(np.uint32), o.fill(0, 2000))


def test_cancel_pending_request_frees_its_place(gpu, orc):
    """A request that waits for budget can be cancelled: its status becomes
    MTGP_ERR_BUSY, its stream is not advanced (it never ran), an admitted
    request cannot be cancelled, and once the budget is released the next
    request on the cancelled one's stream starts where that stream stood."""
    from mtgp_gb300._lib import MTGPError
    from mtgp_gb300.api import Pool, Server
    p = load_table("mtgp32_fast_11213")[0]
    pool = Pool.substreams(p, 1234, 4, jump_table(32))
    start = pool.windows()
    n = 200000
    srv = Server(pool, None, budget_bytes=n * 4 + 4096, slots=2, max_batch=16)
    try:
        a = srv.submit(0, 0, 0, n)              # result kept in the arena
        assert srv.wait(a) == 0
        b = srv.submit(0, 1, 0, n)              # does not fit while a's result is kept
        srv.cancel(b)
        assert srv.wait(b) == -8                # MTGP_ERR_BUSY: cancelled before it ran
        with pytest.raises(MTGPError):
            srv.cancel(a)                       # already done
        got_a = srv.result(a).cpu().numpy().view(np.uint32).copy()
        srv.release(a)                          # the budget is free again
        dst = torch.zeros(n, dtype=torch.int32, device="cuda")
        c = srv.submit(0, 1, 0, n, dst)
        assert srv.wait(c) == 0
        got_c = dst.cpu().numpy().view(np.uint32)
        srv.drain()
    finally:
        srv.close()
    oa, oc = orc.gen(p, seed=1), orc.gen(p, seed=1)
    oa.set_window(start[0])
    oc.set_window(start[1])
    assert np.array_equal(got_a, oa.fill(0, n))
    assert np.array_equal(got_c, oc.fill(0, n))  # stream 1 was not advanced by b
