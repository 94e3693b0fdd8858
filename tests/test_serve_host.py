"""The serving loop's admission rules and output arena
(mtgp_gb300/csrc/server_core.h) on the CPU, through simulated traces: every
request is admitted once; a stream's requests are admitted in submission
order and never while the stream has a batch on the GPU; a long skip only
opens a stream's part of a batch; batches respect max_batch; in-flight
outputs never overlap in the arena nor exceed the budget; all space returns."""
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
    L.probe_serve.argtypes = [ci, vp, vp, vp, vp, ci, ci, ctypes.c_uint64, ci, ci, vp, ci,
                              vp, vp, vp, vp, vp, vp]
    return L


def simulate(probe, pool, stream, skip, nbytes, ns, budget, max_batch, slots, seed):
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
    bret = np.zeros(n + 1, np.int32)
    nb = ctypes.c_int()
    rc = probe.probe_serve(n, p(pool), p(stream), p(skip), p(nbytes), ns[0], ns[1], budget,
                           max_batch, slots, p(retire), len(retire), p(batch), p(off), p(rank),
                           p(badm), p(bret), ctypes.byref(nb))
    return rc, batch, off, rank, badm[:nb.value], bret[:nb.value]


def round256(x):
    return (int(x) + 255) // 256 * 256


@pytest.mark.parametrize("seed", range(6))
def test_admission_invariants(probe, seed):
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
    rc, batch, off, rank, badm, bret = simulate(probe, pool, stream, skip, nbytes, ns, budget,
                                                max_batch, slots, seed)
    assert rc == 0
    assert (batch >= 0).all()
    assert len(set(rank.tolist())) == n
    nb = len(badm)
    assert np.bincount(batch, minlength=nb).max() <= max_batch
    # per stream: submission order == admission order
    for q in (0, 1):
        for s in range(ns[q]):
            idx = np.nonzero((pool == q) & (stream == s))[0]
            assert np.all(np.diff(rank[idx]) > 0)
            # a long skip only as the first of its stream in a batch
            for k in range(1, len(idx)):
                if skip[idx[k]] >= (1 << 17):
                    assert batch[idx[k]] != batch[idx[k - 1]]
    # batches that overlap in time share no stream and no arena bytes
    live = [(badm[b], bret[b]) for b in range(nb)]
    keys = [set(zip(pool[batch == b].tolist(), stream[batch == b].tolist())) for b in range(nb)]
    spans = [[(int(off[k]), int(off[k]) + round256(nbytes[k])) for k in np.nonzero(batch == b)[0]
              if nbytes[k]] for b in range(nb)]
    for a in range(nb):
        for b in range(a + 1, nb):
            if live[a][0] < live[b][1] and live[b][0] < live[a][1]:
                assert not (keys[a] & keys[b])
                for x0, x1 in spans[a]:
                    for y0, y1 in spans[b]:
                        assert x1 <= y0 or y1 <= x0
    for b in range(nb):
        sp = sorted(spans[b])
        assert all(sp[i][1] <= sp[i + 1][0] for i in range(len(sp) - 1))
        assert all(x1 <= budget for _, x1 in sp)


def test_first_come_first_served(probe):
    # a request that does not fit blocks later ones (no overtaking by small
    # requests), until space returns
    pool = [0, 0, 0]
    stream = [0, 1, 2]
    nbytes = [700_000, 700_000, 1000]
    rc, batch, off, rank, badm, bret = simulate(probe, pool, stream, [0, 0, 0], nbytes,
                                                (3, 1), 1 << 20, 8, 4, 0)
    assert rc == 0
    assert batch[0] == 0 and batch[1] == batch[2] == 1


def test_same_stream_shares_a_batch(probe):
    rc, batch, off, rank, badm, bret = simulate(probe, [0] * 4, [5] * 4, [0, 0, 1 << 20, 0],
                                                [100] * 4, (8, 1), 1 << 20, 8, 4, 0)
    assert rc == 0
    assert batch.tolist() == [0, 0, 1, 1]
