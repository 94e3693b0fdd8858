"""The batched-launch planner (mtgp_gb300/csrc/plan_core.cpp) on the CPU:
for random item lists, the tasks it produces step every stream through
exactly the positions the items ask for, write every requested value once
at its offset, generate no long skip when jumps are available, cut long runs
at the chunk length, write each stream's final window back exactly once, and
come longest first (a jump counting as 2^17 values); malformed items are rejected."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from mtgp_gb300._lib import WorkItem

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
JUMP_MIN = 1 << 17


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("plan") / "plan_probe.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", so,
                    os.path.join(HERE, "plan_probe.cpp"),
                    os.path.join(ROOT, "mtgp_gb300", "csrc", "plan_core.cpp")], check=True)
    L = ctypes.CDLL(so)
    vp = ctypes.c_void_p
    L.probe_plan.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                             ctypes.c_int64, ctypes.c_int, vp, ctypes.c_int, vp, ctypes.c_int,
                             vp, ctypes.c_int, vp, ctypes.c_char_p, ctypes.c_int]
    return L


def plan(probe, items, nstreams, word_bytes=4, can_jump=True, chunk=0, resident=100):
    arr = (WorkItem * len(items))()
    for k, (s, kind, count, off, skip) in enumerate(items):
        arr[k].stream, arr[k].kind, arr[k].count, arr[k].out_offset, arr[k].skip = \
            s, kind, count, off, skip
    cap = 4 * len(items) + 64
    while True:
        tc = np.zeros((cap, 7), np.int64)
        sc = np.zeros((cap, 3), np.int64)
        st = np.zeros(cap, np.int32)
        info = np.zeros(6, np.int64)
        err = ctypes.create_string_buffer(256)
        p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        rc = probe.probe_plan(arr, len(items), nstreams, word_bytes, int(can_jump), chunk,
                              resident, p(tc), cap, p(sc), cap, p(st), cap, p(info), err, 256)
        if rc == 1:
            cap = int(max(info[0], info[1], info[2])) + 64
            continue
        if rc:
            return rc, err.value.decode()
        nt, ns, nst = int(info[0]), int(info[1]), int(info[2])
        return 0, (tc[:nt], sc[:ns], st[:nst], int(info[3]), int(info[4]), int(info[5]))


def expected(items, esz):
    """(stream, position) -> (output byte offset, kind) of every output
    value, and each stream's final position."""
    want, end = {}, {}
    for s, kind, count, off, skip in items:
        pos = end.get(s, 0) + skip
        if kind >= 0:
            for i in range(count):
                want[(s, pos + i)] = (off + i * esz, kind)
        end[s] = pos + count
    return want, end


def check(items, res, nstreams, esz, can_jump, chunk_tune):
    tasks, segs, stage, chunk, out_bytes, mode = res
    want, end = expected(items, esz)
    got, ends = {}, {}
    for s, wb, run, off, total, first, n in tasks:
        pos, steps = run + off, 0
        for o, count, kind in segs[first:first + n]:
            if kind >= 0:
                for i in range(count):
                    key = (s, pos + i)
                    assert key not in got, "value produced twice"
                    got[key] = (o + i * esz, kind)
            elif can_jump:
                assert count < JUMP_MIN, "long skip generated although jumps are available"
            pos += count
            steps += count
        assert steps == total
        ends.setdefault(s, []).append((pos, wb))
    assert got == want
    # one write-back per stream, by the task that ends at the stream's end
    for s, e in end.items():
        if e == 0:
            continue
        lst = ends[s]
        writers = [(p, wb) for p, wb in lst if wb != -2]
        assert len(writers) == 1 and writers[0][0] == e, (s, lst, e)
        wb = writers[0][1]
        if len(lst) == 1:
            assert wb == -1
        else:
            assert wb >= 0 and stage[wb] == s
    assert sorted(stage.tolist()) == sorted(set(stage.tolist()))
    jumps = (tasks[:, 2] > 0).astype(np.int64) + (tasks[:, 3] > 0).astype(np.int64)
    cost = tasks[:, 4] + (JUMP_MIN * jumps if can_jump else 0)
    assert np.all(cost[:-1] >= cost[1:]), "not longest first"
    assert not can_jump or chunk_tune >= 0 or chunk == 0
    if chunk_tune > 0 and chunk:
        assert chunk == chunk_tune
    if chunk:
        # pieces of a cut run: near-equal, a multiple of the grain (largest
        # power of two <= chunk / 8, at most 2^16), at most chunk + grain,
        # the last taking the rest; uncut runs are at most one chunk
        grain = 1
        while grain * 2 <= chunk // 8 and grain < (1 << 16):
            grain *= 2
        by_run = {}
        for s, wb, run, off, total, first, n in tasks:
            by_run.setdefault((s, run), []).append((off, total))
        for pieces in by_run.values():
            pieces.sort()
            if len(pieces) > 1:
                piece = pieces[0][1]
                assert piece % grain == 0 and piece < chunk + grain
                assert all(t == piece for _, t in pieces[:-1])
                assert 0 <= pieces[-1][1] <= piece
                assert [o for o, _ in pieces] == [k * piece for k in range(len(pieces))]
    ob = max([off + count * esz for s, kind, count, off, skip in items if kind >= 0 and count],
             default=0)
    assert out_bytes == ob


def random_items(rng, nstreams, nitems, esz, big):
    items, off = [], 0
    for _ in range(nitems):
        s = int(rng.integers(0, nstreams))
        kind = int(rng.integers(-1, 5))
        count = int(rng.integers(0, 3000))
        if rng.random() < 0.1:
            count = int(rng.integers(3000, 20000))
        skip = 0
        u = rng.random()
        if u < 0.15:
            skip = int(rng.integers(1, 3000))
        elif u < 0.25 and big:
            skip = int(rng.integers(JUMP_MIN, 3 * JUMP_MIN))
        items.append((s, kind, count, off, skip))
        if kind >= 0:
            off += count * esz
    return items


@pytest.mark.parametrize("can_jump", [True, False])
@pytest.mark.parametrize("chunk", [0, -1, 1000, 4096])
@pytest.mark.parametrize("esz", [4, 8])
def test_plan_matches_model(probe, can_jump, chunk, esz):
    rng = np.random.default_rng(11 + chunk + esz + can_jump)
    for trial in range(6):
        nstreams = int(rng.integers(1, 12))
        items = random_items(rng, nstreams, int(rng.integers(1, 40)), esz, big=can_jump)
        rc, res = plan(probe, items, nstreams, esz, can_jump, chunk, resident=4)
        assert rc == 0, res
        check(items, res, nstreams, esz, can_jump, chunk)


def test_plan_advance_only_and_trailing_jump(probe):
    # an advance-only item longer than the jump threshold becomes a jump; a
    # stream that ends with a jump still gets a task that writes its window
    items = [(0, 0, 10, 0, 0), (0, -1, 3 * JUMP_MIN, 0, 0), (0, 1, 5, 40, 0),
             (1, -1, 0, 0, 5 * JUMP_MIN)]
    rc, res = plan(probe, items, 2)
    assert rc == 0, res
    tasks, segs = res[0], res[1]
    check(items, res, 2, 4, True, 0)
    t1 = [t for t in tasks if t[0] == 1]
    assert len(t1) == 1 and t1[0][2] == 5 * JUMP_MIN and t1[0][1] == -1
    assert len([t for t in tasks if t[0] == 0]) == 2   # the run after the jump


def test_plan_rejects_bad_items(probe):
    assert plan(probe, [(3, 0, 10, 0, 0)], 2)[0] == -2          # stream out of range
    assert plan(probe, [(0, 7, 10, 0, 0)], 2)[0] == -2          # unknown kind
    assert plan(probe, [(0, 0, 10, 2, 0)], 2)[0] == -2          # misaligned offset
    assert plan(probe, [(0, 0, 10, 0, 1 << 35)], 2, can_jump=False)[0] == -3  # huge generated skip
    assert plan(probe, [(0, 0, 10, 0, 1 << 35)], 2, can_jump=True)[0] == 0
    assert plan(probe, [(0, 0, 1, 0, (1 << 64) - 1), (0, 0, 1, 4, 5)], 2)[0] == -2  # overflow


def test_plan_automatic_chunk(probe):
    # chunk = next power of two >= generated values / resident, at least 2^17;
    # reported only when some run was cut
    items = [(s, 0, 300_000, 1_200_000 * s, 0) for s in range(4)]
    rc, res = plan(probe, items, 4, resident=2)
    assert rc == 0 and res[3] == 0 and len(res[0]) == 4   # 2^20 chunks: nothing to cut
    rc, res = plan(probe, items, 4, resident=8)
    assert rc == 0 and res[3] == 1 << 18   # 150 k per slot -> 2^18 < 300 k: two pieces
    assert len(res[0]) == 8 and set(res[0][:, 4].tolist()) == {163840, 136160}  # grain 2^15
    check(items, res, 4, 4, True, 0)
    rc, res = plan(probe, items, 4, resident=16)
    assert rc == 0 and res[3] == 1 << 17                   # 75 k per slot -> 2^17, cut
    check(items, res, 4, 4, True, 0)
    rc, res = plan(probe, items + [(4, 0, 5_000_000, 4_800_000, 0)], 5, resident=64)
    assert rc == 0 and res[3] == 1 << 17
    check(items + [(4, 0, 5_000_000, 4_800_000, 0)], res, 5, 4, True, 0)


def test_jump_part_chunks(probe):
    """Every tap chunk of a jump goes to exactly one part, no part is empty,
    and the earlier parts (which generate less of the sequence) take the
    extra chunks."""
    import ctypes
    probe.probe_part_chunks.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    for tch in range(1, 64):
        for parts in range(1, tch + 1):
            b = np.zeros(parts + 1, np.int32)
            probe.probe_part_chunks(tch, parts, b.ctypes.data_as(ctypes.c_void_p))
            sizes = np.diff(b)
            assert b[0] == 0 and b[-1] == tch and (sizes > 0).all(), (tch, parts, b)
            assert (np.diff(sizes) <= 0).all(), (tch, parts, sizes)
    b = np.zeros(5, np.int32)
    probe.probe_part_chunks(11, 4, b.ctypes.data_as(ctypes.c_void_p))
    assert b.tolist() == [0, 3, 6, 9, 11]
