"""The serving loop's admission rules, stream order and output arena
(mtgp_gb300/csrc/server_core.h) on the CPU, through simulated traces: every
request is admitted once; a stream's requests are admitted in submission
order; a batch holding a stream whose earlier batch is still in flight is
ordered after that batch; a long skip only opens a stream's part of a batch;
batches respect max_batch and an eighth of the budget; blocks are placed in
admission order; in-flight outputs never overlap in the arena nor exceed the
budget; all space returns."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("serve") / "serve_probe.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", so,
                    os.path.join(HERE, "serve_probe.cpp")], check=True)
    L = ctypes.CDLL(so)
    vp, ci = ctypes.c_void_p, ctypes.c_int
    L.probe_batch_cap.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int]
    L.probe_batch_bytes.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
    L.probe_batch_bytes.restype = ctypes.c_uint64
    L.probe_serve.argtypes = [ci, vp, vp, vp, vp, ci, ci, ctypes.c_uint64, ci, ci, ci, vp,
                              ci, vp, vp, vp, vp, vp, vp, vp, vp]
    return L


def simulate(probe, pool, stream, skip, nbytes, ns, budget, max_batch, slots, seed,
             pipe_backlog=0):
    n = len(pool)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    pool = np.ascontiguousarray(pool, np.int32)
    stream = np.ascontiguousarray(stream, np.uint32)
    skip = np.ascontiguousarray(skip, np.uint64)
    nbytes = np.ascontiguousarray(nbytes, np.uint64)
    retire = np.random.default_rng(seed).integers(0, 1 << 30, 4096).astype(np.uint32)
    batch = np.full(n, -1, np.int32)
    off = np.zeros(n, np.uint64)
    rank = np.full(n, -1, np.int32)
    badm = np.zeros(n + 1, np.int32)
    bplc = np.zeros(n + 1, np.int32)
    bret = np.zeros(n + 1, np.int32)
    deps = np.full((n + 1) * slots, -1, np.int32)
    nb = ctypes.c_int()
    rc = probe.probe_serve(n, p(pool), p(stream), p(skip), p(nbytes), ns[0], ns[1], budget,
                           max_batch, slots, pipe_backlog, p(retire), len(retire), p(batch),
                           p(off), p(rank),
                           p(badm), p(bplc), p(bret), p(deps), ctypes.byref(nb))
    m = nb.value
    return dict(rc=rc, batch=batch, off=off, rank=rank, admit=badm[:m], place=bplc[:m],
                retire=bret[:m], deps=[set(d[d >= 0].tolist()) for d in deps[:m * slots]
                                       .reshape(m, slots)] if m else [])


def round256(x):
    return (int(x) + 255) // 256 * 256


@pytest.mark.parametrize("pipe_backlog", [0, 100, 1 << 30])
@pytest.mark.parametrize("seed", range(6))
def test_admission_invariants(probe, seed, pipe_backlog):
    rng = np.random.default_rng(seed)
    n = 600
    ns = (int(rng.integers(1, 40)), int(rng.integers(1, 8)))
    pool = (rng.random(n) < 0.2).astype(np.int32)
    stream = np.where(pool == 0, rng.integers(0, ns[0], n), rng.integers(0, ns[1], n))
    skip = np.where(rng.random(n) < 0.15, 1 << 20, np.where(rng.random(n) < 0.2, 100, 0))
    nbytes = rng.integers(0, 200_000, n)
    nbytes[rng.random(n) < 0.05] = 0
    budget = 1 << 20
    max_batch = int(rng.integers(1, 64))
    slots = int(rng.integers(1, 5))
    r = simulate(probe, pool, stream, skip, nbytes, ns, budget, max_batch, slots, seed,
                 pipe_backlog)
    assert r["rc"] == 0
    batch, off, rank = r["batch"], r["off"], r["rank"]
    assert (batch >= 0).all()
    assert len(set(rank.tolist())) == n
    nb = len(r["admit"])
    assert np.bincount(batch, minlength=nb).max() <= max_batch
    # blocks are placed in admission order
    assert np.all(np.diff(r["place"]) >= 0)
    assert np.all(r["place"] >= r["admit"]) and np.all(r["retire"] > r["place"])
    for q in (0, 1):
        for s in range(ns[q]):
            idx = np.nonzero((pool == q) & (stream == s))[0]
            # per stream: submission order == admission order
            assert np.all(np.diff(rank[idx]) > 0)
            for k in range(1, len(idx)):
                a, b = batch[idx[k - 1]], batch[idx[k]]
                # a long skip only as the first of its stream in a batch
                if skip[idx[k]] >= (1 << 17):
                    assert a != b
                # a later batch of the stream runs after the earlier one: it
                # was retired before the later one was admitted, or the
                # later one is ordered after it
                if a != b:
                    assert a < b
                    assert r["retire"][a] < r["admit"][b] or a in r["deps"][b]
                    assert r["retire"][a] < r["retire"][b]
                    if pipe_backlog > n:  # never pipelined: one batch of a stream at a time
                        assert r["retire"][a] < r["admit"][b]
    spans = [[(int(off[k]), int(off[k]) + round256(nbytes[k])) for k in np.nonzero(batch == b)[0]
              if nbytes[k]] for b in range(nb)]
    for b in range(nb):
        sp = sorted(spans[b])
        assert all(sp[i][1] <= sp[i + 1][0] for i in range(len(sp) - 1))
        assert all(x1 <= budget for _, x1 in sp)
        # at most an eighth of the budget, unless the batch is one request
        size = sum(x1 - x0 for x0, x1 in sp)
        assert size <= budget // 8 or len(sp) == 1
    # batches in the arena at the same time share no bytes
    for a in range(nb):
        for b in range(a + 1, nb):
            if r["place"][a] < r["retire"][b] and r["place"][b] < r["retire"][a]:
                for x0, x1 in spans[a]:
                    for y0, y1 in spans[b]:
                        assert x1 <= y0 or y1 <= x0


def test_first_come_first_served(probe):
    # a batch whose block does not fit holds back later ones (no overtaking by
    # small requests) until space returns; a batch takes at most an eighth of
    # the budget unless it is one request
    r = simulate(probe, [0, 0, 0], [0, 1, 2], [0, 0, 0], [700_000, 700_000, 1000], (3, 1),
                 1 << 20, 8, 4, 0)
    assert r["rc"] == 0
    assert r["batch"].tolist() == [0, 1, 2]
    assert r["place"][1] > r["retire"][0] and r["place"][2] >= r["place"][1]


def test_same_stream_shares_a_batch(probe):
    r = simulate(probe, [0] * 4, [5] * 4, [0, 0, 1 << 20, 0], [100] * 4, (8, 1), 1 << 20, 8,
                 4, 0)
    assert r["rc"] == 0
    assert r["batch"].tolist() == [0, 0, 1, 1]


def test_stream_in_flight_waits_without_backlog(probe):
    # the same trace without a backlog: the stream's second request waits for
    # its first batch, and the other stream's request goes ahead of it
    r = simulate(probe, [0, 0, 0], [3, 3, 4], [0, 0, 0], [100, 100, 100], (8, 1), 1 << 20, 1,
                 4, 0, pipe_backlog=1 << 30)
    assert r["rc"] == 0
    assert r["batch"].tolist() == [0, 2, 1]
    assert r["admit"][2] > r["retire"][0]
    assert r["deps"] == [set(), set(), set()]


def test_stream_in_flight_joins_the_next_batch(probe):
    # one request per batch: the stream's second request is admitted while its
    # first batch is in flight and ordered after it; another stream's is not
    r = simulate(probe, [0, 0, 0], [3, 3, 4], [0, 0, 0], [100, 100, 100], (8, 1), 1 << 20, 1,
                 4, 0)
    assert r["rc"] == 0
    assert r["batch"].tolist() == [0, 1, 2]
    assert r["admit"][1] < r["retire"][0]
    assert r["deps"] == [set(), {0}, set()]
    assert r["retire"][1] > r["retire"][0]


def test_batch_cap(probe):
    cap = probe.probe_batch_cap
    assert cap(5, 8192, 0) == 8192            # no backlog: max_batch
    assert cap(100000, 8192, 1) == 8192       # a burst: full batches
    assert cap(20000, 8192, 1) == 5000        # near capacity: a quarter of what waits
    assert cap(6000, 8192, 1) == 2048         # at least a quarter of max_batch
    assert cap(1, 1, 1) == 1 and cap(0, 2, 1) == 1  # never zero


def test_batch_bytes(probe):
    nb = probe.probe_batch_bytes
    gb = 1 << 30
    assert nb(0, 8 * gb) == gb                # a light load: an eighth of the arena
    assert nb(16 * gb, 8 * gb) == 2 * gb      # a backlog: an eighth of what waits
    assert nb(100 * gb, 8 * gb) == 4 * gb     # a burst: at most half the arena
