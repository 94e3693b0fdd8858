"""Benchmark of the GB300 MTGP generator.

Workload (the batched configuration the headline metric is quoted on):
MTGP32-11213 parameter set 0 (mtgp32_params_fast_11213[0]), seed 1234,
4096 substreams, substream j starting j * 3^162 steps ahead (jumped on the
GPU with the reference's jump table), and per substream a request of
lognormal length (median 2^16 uint32, sigma 1.0, seed 42, clipped to
[2^10, 2^22]) -- about 1.8 GB of output per step.  A step generates every
substream's request once (states advance from step to step).

Reported (one JSON line on rank 0):
  value     batched GB/s of output, device-resident, one persistent launch
            per step replayed from a CUDA graph, CUDA-event timed
  e2e       the same through the C ABI from host data: the work items are
            uploaded and the whole output is read back to pinned host memory
            every step
  plain     the same workload with one launch (one CTA) per substream
  bank      128-set bank (2^21 uint32 per set, one CTA per set) GB/s
  roofline  batched kernel vs the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (OpenMP over substreams) on a sample
  serve     continuous-batching server over resident streams: saturation
            rate, then p50 / p99 latency and GB/s at 0.3 / 0.6 / 0.9 of it;
            a check trace whose every response is compared with the oracle

    python bench.py [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import ctypes
import json
import os

# the concurrent plain leg spreads its launches over 32 CUDA streams; give
# each its own hardware queue (read when the CUDA context is created)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_SUB = 4096
SEED = 1234
L2_BYTES = 129 * 2 ** 20
# DRAM bytes per step of the batched plan's kernels, from one ncu capture
# of one launch each (dram__bytes_read.sum + dram__bytes_write.sum), keyed
# by the captured plan's (core, split chunk, grid, windows jumped ahead)
CAPTURED_TRAFFIC = {
    (2, 393216, 760, 184): {
        "bytes": 1677.8e6 + 6.85e6 + 0.52e6,
        "source": "ncu capture of k_batch32xk<2> + k_jump_part5, one launch each, this plan "
                  "(profiles/bench_default_plan_k_batch32xk2_k_jump_part5.md)"},
}
METRIC = "batched MTGP32-11213 output GB/s"
WORKLOAD = ("batched: mtgp32_params_fast_11213[0], seed 1234, 4096 substreams j*3^162 "
            "(GPU jump), lognormal lengths median 2^16 sigma 1.0 seed 42 clip [2^10,2^22], uint32")


SERVE_WORKLOAD = ("serving: 4096 MTGP32-11213 substreams (set 0) + 256 MTGP64-11213 substreams "
                  "(mtgp64dc set 0), j*3^162 apart, seed 1234; Poisson arrivals; stream uniform; "
                  "count lognormal median 2^16 sigma 1.0 clip [1,2^26]; types uint32 / float32 "
                  "[0,1) / uint64 60/30/10; 10% of requests at an offset 2^k, k uniform in "
                  "17..40 (GF(2) jump on the GPU); 8 GB device budget for in-flight output")


def serve_trace(rng, n):
    """n requests of the serving workload: (pool, stream, kind, count, skip)."""
    u = rng.random(n)
    pool = (u >= 0.9).astype(np.int32)
    kind = np.where((u >= 0.6) & (u < 0.9), 2, 0).astype(np.int32)
    stream = np.where(pool == 0, rng.integers(0, 4096, n), rng.integers(0, 256, n))
    count = np.clip(np.rint(rng.lognormal(np.log(2.0 ** 16), 1.0, n)), 1, 2 ** 26)
    skip = np.where(rng.random(n) < 0.1, np.left_shift(1, rng.integers(17, 41, n)), 0)
    return pool, stream.astype(np.uint32), kind, count.astype(np.uint64), skip.astype(np.uint64)


def replica_seed(rank):
    """Replicas are independent jobs: rank r seeds its substreams with
    SEED + r, so no two ranks produce the same numbers."""
    return SEED + rank


def max_over_ranks(x, world, device="cuda"):
    """The slowest rank's time (the job ends when its last rank does)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world, bytes_per_rank, ms):
    """Whole-job GB/s: every rank's output over the slowest rank's time."""
    return world * bytes_per_rank / (ms * 1e-3) / 1e9


def lengths(n=N_SUB, seed=42):
    rng = np.random.default_rng(seed)
    x = rng.lognormal(mean=np.log(2.0 ** 16), sigma=1.0, size=n)
    return np.clip(np.rint(x), 2 ** 10, 2 ** 22).astype(np.int64)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampler running while the GPU is busy."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, dev=0):
        self.p = None
        self.dev = dev

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        self.rows = []
        if self.p is None:
            return
        time.sleep(0.15)
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except Exception:
            self.p.kill()
            out = ""
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 7:
                self.rows.append(f)

    def summary(self):
        rows = getattr(self, "rows", [])
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def cpu_baseline(orc, params, windows, lens, sample_streams, gpu_first_step, min_seconds=10.0):
    """Oracle (port of the reference, OpenMP over streams) on a sample of the
    workload, repeated until min_seconds of wall time; returns GB/s.  Its
    first repetition is also the checker of the GPU's first step for the
    sampled substreams (bit-exact)."""
    from mtgp_gb300.params import params_array, MTGP32Params
    parr = params_array(MTGP32Params, [params])
    win = np.ascontiguousarray(windows[:sample_streams].copy())
    counts = lens[:sample_streams].astype(np.uint64)
    offs = (np.concatenate([[0], np.cumsum(counts)[:-1]]) * 4).astype(np.uint64)
    out = np.empty(int(counts.sum()), dtype=np.uint32)
    kinds = np.zeros(sample_streams, np.int32)
    pidx = np.zeros(sample_streams, np.int32)
    reps, t0 = 0, time.perf_counter()
    while True:
        orc.multi_fill(32, parr, win, counts, kinds, offs, out, param_idx=pidx)
        if reps == 0:
            verified = bool(np.array_equal(out, gpu_first_step[:out.size]))
            assert verified, "GPU output differs from the oracle"
            t0 = time.perf_counter()
        reps += 1
        dt = time.perf_counter() - t0
        if dt >= min_seconds and reps > 1:
            break
    return (reps - 1) * out.nbytes / dt / 1e9, reps - 1, int(counts.sum()), verified


def run_reference(args):
    """--impl reference: the reference's CPU code on the host cores, OpenMP
    over substreams, on a bounded sample of the same workload per step."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from mtgp_gb300.params import jump_table, load_table
    lens = lengths()
    p = load_table("mtgp32_fast_11213")[0]
    sample = 256
    from oracle.bind import Oracle, build
    build()
    orc = Oracle()
    # substream start states (the reference's own jump on the CPU)
    g = orc.gen(p, seed=SEED)
    from mtgp_gb300.params import jump_string
    js = jump_string(32)
    wins = []
    for j in range(sample):
        wins.append(g.window())
        g.fast_jump(js)
    wins = np.stack(wins)
    counts = lens[:sample].astype(np.uint64)
    offs = (np.concatenate([[0], np.cumsum(counts)[:-1]]) * 4).astype(np.uint64)
    out = np.empty(int(counts.sum()), dtype=np.uint32)
    from mtgp_gb300.params import params_array, MTGP32Params
    parr = params_array(MTGP32Params, [p])
    cores = orc.max_threads()
    times = []
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        orc.multi_fill(32, parr, wins, counts, np.zeros(sample, np.int32), offs, out,
                       param_idx=np.zeros(sample, np.int32))
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            times.append(dt)
    value = out.nbytes * len(times) / sum(times) / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3),
        "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * sum(times) / len(times), 3), "higher_is_better": True,
        "dtype": "u32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample": "first %d substreams per step" % sample},
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": cores,
                         "kind": "port",
                         "sample": "first %d substreams (%d uint32) per step" % (sample, out.size)},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_serving(args, s, local):
    """Serving section: a check trace, a burst that finds the saturation
    rate, then Poisson traces at 0.3 / 0.6 / 0.9 of it with p50 / p99
    latency (submission to the result resident in device memory).  Every
    request submitted is recorded in order, so that the oracle can place any
    of them in its stream; from each timed trace a sample of requests (of
    each output type, the trace's largest, and one planted request of 2^25 +
    12345 uint32 plus one of 2^24 + 7 uint64 after a jumped offset) gets a
    device destination and is checked afterwards."""
    import torch
    from mtgp_gb300.api import Pool, Server, requests
    from mtgp_gb300.params import jump_table, load_table
    # the library's default planning: the pools below take the process
    # defaults (the batched section tuned its own pool only)
    p32 = load_table("mtgp32_fast_11213")[0]
    p64 = load_table("mtgp64dc_fast_11213")[0]
    a = Pool.substreams(p32, SEED, 4096, jump_table(32), stream=s)
    b = Pool.substreams(p64, SEED, 256, jump_table(64), stream=s)
    s.synchronize()
    win_a, win_b = a.windows(), b.windows()
    srv = Server(a, b, budget_bytes=8 << 30, slots=args.serve_slots, max_batch=8192)
    history = []          # every request submitted, in submission order
    samples = []          # (index in history, host output)
    # check trace: every response kept for the bit-exact check on the CPU
    rng = np.random.default_rng(7)
    pool, stream, kind, count, skip = serve_trace(rng, 256)
    count = np.minimum(count, 1 << 18)
    outs = []
    for k in range(256):
        dst = torch.empty(int(count[k]), dtype=torch.int32 if pool[k] == 0 else torch.int64,
                          device="cuda")
        outs.append(dst)
        srv.submit(int(pool[k]), int(stream[k]), int(kind[k]), int(count[k]), dst,
                   skip=int(skip[k]))
    srv.drain()
    base = len(history)
    history.extend(zip(pool, stream, kind, count, skip))
    samples.extend((base + k, outs[k].cpu().numpy()) for k in range(256))
    del outs

    def run(tr, arrivals, sample=0):
        req = requests(*tr)
        picked, bufs = [], []
        if sample:
            n = len(req)
            # planted long requests: above 2^24 values, uint32 and uint64
            req[n // 2] = (0, req[n // 2]["stream"] % 4096, 0, 0, 0, (1 << 25) + 12345, 0)
            req[n // 3] = (1, req[n // 3]["stream"] % 256, 0, 0, 1 << 20, (1 << 24) + 7, 0)
            picked = {n // 2, n // 3, int(np.argmax(req["count"]))}
            for pool_, kind_ in ((0, 0), (0, 2), (1, 0)):
                idx = np.flatnonzero((req["pool"] == pool_) & (req["kind"] == kind_))
                picked.update(int(x) for x in rng.choice(idx, min(sample, idx.size), False))
            picked = sorted(picked)
            for k in picked:
                dt = torch.int32 if req[k]["pool"] == 0 else torch.int64
                d = torch.empty(int(req[k]["count"]), dtype=dt, device="cuda")
                bufs.append(d)
                req["dst"][k] = d.data_ptr()
        c0, b0, k0 = srv.stats()
        wall = srv.replay(req, arrivals)
        c1, b1, k1 = srv.stats()
        lat, st = srv.results()
        assert (st[c0:c1] == 0).all(), "failed requests"
        base = len(history)
        history.extend(zip(req["pool"], req["stream"], req["kind"], req["count"], req["skip"]))
        samples.extend((base + k, d.cpu().numpy()) for k, d in zip(picked, bufs))
        return wall, b1 - b0, k1 - k0, lat[c0:c1]

    rng = np.random.default_rng(11)
    # warm-up: plan buffers, kernels, the jump polynomials of the offsets and
    # of the chunk multiples
    for n in (2000, args.serve_burst):
        run(serve_trace(rng, n), np.zeros(n))
    run(serve_trace(rng, 20000), np.cumsum(rng.exponential(1e-6, 20000)))
    out = {"workload": SERVE_WORKLOAD, "slots": args.serve_slots, "max_batch": 8192,
           "latency": "submission to the result resident in device memory"}
    with Clocks(local) as clk:
        n = args.serve_burst
        wall, nbytes, batches, lat = run(serve_trace(rng, n), np.zeros(n), args.serve_sample)
        sat = n / wall
        out["saturation"] = {"requests": n, "req_per_s": round(sat, 1),
                             "GB_per_s": round(nbytes / wall / 1e9, 2), "batches": batches}
        rates = []
        for load in (0.3, 0.6, 0.9):
            rate = load * sat
            n = max(200, int(rate * args.serve_seconds))
            arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
            wall, nbytes, batches, lat = run(serve_trace(rng, n), arrivals, args.serve_sample)
            rates.append({"load": load, "offered_req_per_s": round(rate, 1), "requests": n,
                          "req_per_s": round(n / wall, 1),
                          "GB_per_s": round(nbytes / wall / 1e9, 2),
                          "p50_ms": round(1e3 * float(np.percentile(lat, 50)), 3),
                          "p99_ms": round(1e3 * float(np.percentile(lat, 99)), 3),
                          "batches": batches})
        out["rates"] = rates
    out["clocks"] = clk.summary()
    out["scheduler_s"] = {k: round(v, 3) for k, v in srv.profile().items()}
    srv.close()
    return out, (history, samples, win_a, win_b)


POLY_WORKLOAD = ("jump polynomials X^e mod chi of mtgp32_params_fast_11213[0] on the GPU, "
                 "e uniform in [2^56, 2^63)")


def run_polys(args, s):
    """Jump-polynomial section: X^e mod chi for arbitrary 64-bit exponents
    computed on the GPU (byte-window tables, then products).  Latency of one
    exponent through the public call (host exponent in, device polynomial
    out) and throughput of args.poly_n exponents per call."""
    import torch
    from mtgp_gb300.api import Pool
    from mtgp_gb300.params import load_table
    p = load_table("mtgp32_fast_11213")[0]
    pool = Pool.create([p], [SEED], [0])
    t0 = time.perf_counter()
    pool.jump_polys(0, [12345], stream=s)  # tables: characteristic polynomial, X^(k 2^(8m))
    s.synchronize()
    table_ms = (time.perf_counter() - t0) * 1e3
    rng = np.random.default_rng(13)
    lat = []
    for _ in range(3 + args.poly_reps):
        e = int(rng.integers(1 << 56, 1 << 63))
        t0 = time.perf_counter()
        pool.jump_polys(0, [e], stream=s)
        s.synchronize()
        lat.append(time.perf_counter() - t0)
    lat = np.array(lat[3:])
    st = rng.integers(1 << 56, 1 << 63, args.poly_n, dtype=np.int64)
    pool.jump_polys(0, st, stream=s)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.synchronize()
    t0 = time.perf_counter()
    ev0.record(s)
    for _ in range(args.poly_reps):
        pool.jump_polys(0, st, stream=s)
    ev1.record(s)
    s.synchronize()
    wall = (time.perf_counter() - t0) / args.poly_reps
    dev_ms = ev0.elapsed_time(ev1) / args.poly_reps
    return {"workload": POLY_WORKLOAD, "table_setup_ms": round(table_ms, 2),
            "one_exponent_ms": {"p50": round(1e3 * float(np.percentile(lat, 50)), 3),
                                "p99": round(1e3 * float(np.percentile(lat, 99)), 3),
                                "calls": int(lat.size)},
            "batch": {"exponents": int(args.poly_n), "ms": round(wall * 1e3, 3),
                      "device_ms": round(dev_ms, 3),
                      "per_s": round(args.poly_n / wall, 1)}}


def run_single(s, reps=50):
    """One generator (mtgp32_params_fast_11213[0], seed 1234): 2^20 uint32
    then 2^20 float32 in [1,2) per step into device memory, through the
    generator's fill calls (each fill split over many CTAs from chunk
    windows jumped ahead on the GPU)."""
    import torch
    from mtgp_gb300.api import MTGP32
    from mtgp_gb300.params import load_table
    g = MTGP32(load_table("mtgp32_fast_11213")[0], seed=1234)
    n = 1 << 20
    out = torch.empty(2 * n, dtype=torch.int32, device="cuda")
    flt = out[n:].view(torch.float32)

    def step():
        g.fill_into(0, out[:n], n, stream=s)
        g.fill_into(1, flt, n, stream=s)
    for _ in range(5):
        step()
    s.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(s)
    for _ in range(reps):
        step()
    ev1.record(s)
    s.synchronize()
    ms = ev0.elapsed_time(ev1) / reps
    return {"workload": "one generator, mtgp32_params_fast_11213[0] seed 1234: 2^20 uint32 "
                        "then 2^20 float32 [1,2) per step, device output",
            "value": round(2 * n * 4 / (ms * 1e-3) / 1e9, 2), "unit": "GB/s",
            "ms_per_step": round(ms, 4), "steps": reps}


def poly_cpu_baseline(orc, seconds):
    """The oracle's bit-serial PowerXMod (one core) on the same exponents'
    distribution: polynomials per second over a bounded sample."""
    from mtgp_gb300.params import load_table
    p = load_table("mtgp32_fast_11213")[0]
    seq = orc.gen(p, seed=1).fill(0, 2 * p.mexp)
    d, chi = orc.minpoly((seq & 1).astype(np.uint8))
    rng = np.random.default_rng(13)
    n, t0 = 0, time.perf_counter()
    while n < 2 or (time.perf_counter() - t0 < seconds and n < 64):
        orc.powxmod(int(rng.integers(1 << 56, 1 << 63)), chi, d)
        n += 1
    dt = time.perf_counter() - t0
    return {"value": round(n / dt, 2), "unit": "polynomials/s", "cores": 1, "kind": "port",
            "sample": "%d exponents, bit-serial PowerXMod" % n}


def full_check(orc, p, start_windows, lens, first_step, last_step, end_windows, nsteps):
    """Every substream of the first and of the last timed step against the
    oracle (OpenMP over substreams): the oracle replays all nsteps launches
    from the substreams' start windows, and the outputs of launch 1 and
    launch nsteps are compared word for word, then the windows after launch
    nsteps (word 0 under the state mask, as the reference's own check does,
    cuda-sample/mtgp32-sample-jump1-host.cu:100-108)."""
    from mtgp_gb300.params import MTGP32Params, params_array
    n = len(lens)
    parr = params_array(MTGP32Params, [p])
    win = np.ascontiguousarray(start_windows.copy())
    counts = lens.astype(np.uint64)
    offs = (np.concatenate([[0], np.cumsum(lens)[:-1]]) * 4).astype(np.uint64)
    ref = np.empty(int(lens.sum()), dtype=np.uint32)
    zeros = np.zeros(n, np.int32)
    t0 = time.perf_counter()
    res = {"substreams": n, "launches_replayed": nsteps}

    def bad_streams(got):
        return [j for j in range(n) if not np.array_equal(
            got[offs[j] // 4:offs[j] // 4 + counts[j]], ref[offs[j] // 4:offs[j] // 4 + counts[j]])]

    for k in range(1, nsteps + 1):
        orc.multi_fill(32, parr, win, counts, zeros, offs, ref, param_idx=zeros)
        if k == 1:
            res["first_step_mismatched_substreams"] = len(bad_streams(first_step))
        if k == nsteps:
            res["last_step_mismatched_substreams"] = len(bad_streams(last_step))
    w0 = ((end_windows[:, 0] ^ win[:, 0]) & np.uint32(p.mask)) == 0
    res["final_windows_mismatched"] = int((~(w0 & (end_windows[:, 1:] == win[:, 1:]).all(1))).sum())
    res["bit_exact"] = (res["first_step_mismatched_substreams"] == 0
                        and res["last_step_mismatched_substreams"] == 0
                        and res["final_windows_mismatched"] == 0)
    res["oracle_s"] = round(time.perf_counter() - t0, 2)
    return res


def cpu_rate(orc, bits, plist, pidx, windows, counts, kinds, seconds):
    """The oracle (OpenMP over streams) on a sample of a bank workload,
    repeated for about `seconds`: GB/s of output."""
    from mtgp_gb300.params import MTGP32Params, MTGP64Params, params_array
    parr = params_array(MTGP32Params if bits == 32 else MTGP64Params, plist)
    win = np.ascontiguousarray(windows.copy())
    counts = np.ascontiguousarray(counts, np.uint64)
    esz = bits // 8
    offs = (np.concatenate([[0], np.cumsum(counts)[:-1]]) * esz).astype(np.uint64)
    out = np.empty(int(counts.sum()) * esz, dtype=np.uint8)
    reps, t0 = 0, time.perf_counter()
    while reps < 2 or time.perf_counter() - t0 < seconds:
        orc.multi_fill(bits, parr, win, counts, np.asarray(kinds, np.int32), offs, out,
                       param_idx=np.asarray(pidx, np.int32))
        reps += 1
    dt = time.perf_counter() - t0
    return round(reps * out.nbytes / dt / 1e9, 3), reps, out.nbytes


def write_peak(reps=10):
    """Store-only HBM bandwidth: a 4 GiB buffer written by torch's fill
    kernel, best of `reps` (CUDA events); the roofline's copy peak counts a
    read and a write per byte, this one writes only."""
    import torch
    buf = torch.empty(1 << 30, dtype=torch.int32, device="cuda")
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = None
    for r in range(reps + 2):
        ev0.record()
        buf.fill_(r)
        ev1.record()
        ev1.synchronize()
        if r >= 2:
            ms = ev0.elapsed_time(ev1)
            best = ms if best is None else min(best, ms)
    del buf
    return round(4 * (1 << 30) / (best * 1e-3) / 1e9, 1)


def plain_concurrent(pool, lens, offs, out, nstreams=32, steps=3):
    """The plain one-launch-per-substream path (one CTA each, as the
    reference's sample launches one block per generator) with the launches
    dealt round-robin to `nstreams` CUDA streams, so that many CTAs run at
    once, captured once into a CUDA graph (no host launch cost) and replayed:
    ms per step."""
    import torch
    n = len(lens)
    s0 = torch.cuda.Stream()
    streams = [torch.cuda.Stream() for _ in range(nstreams)]

    def issue():
        ev = torch.cuda.Event()
        ev.record(s0)
        for st in streams:
            st.wait_event(ev)
        for j in range(n):
            pool.fill_stream(j, 0, out, int(lens[j]), stream=streams[j % nstreams],
                             byte_offset=int(offs[j]))
        for st in streams:
            e = torch.cuda.Event()
            e.record(st)
            s0.wait_event(e)

    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s0):
        issue()
    g.replay()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(s0):
        ev0.record(s0)
        for _ in range(steps):
            g.replay()
        ev1.record(s0)
    s0.synchronize()
    return ev0.elapsed_time(ev1) / steps


def serve_check(orc, chk):
    """The sampled responses against the oracle.  A request's values start
    at its stream's position when it is served: the sum of skip + count of
    every earlier request on that stream, in submission order, plus its own
    skip.  The oracle goes there from the stream's start window by X^position
    mod chi when that is 2^17 or more (its bit-serial PowerXMod; the same
    values as stepping), else by stepping, and fills."""
    from mtgp_gb300.params import load_table
    history, samples, win_a, win_b = chk
    par = {0: load_table("mtgp32_fast_11213")[0], 1: load_table("mtgp64dc_fast_11213")[0]}
    chis = {}
    for q, p in par.items():
        seq = orc.gen(p, seed=1).fill(0, 2 * p.mexp)
        chis[q] = orc.minpoly((seq & 1).astype(np.uint8))
    want = {k: o for k, o in samples}
    pos, where = {}, {}
    for k, (q, j, kind, count, skip) in enumerate(history):
        key = (int(q), int(j))
        start = pos.get(key, 0) + int(skip)
        pos[key] = start + int(count)
        if k in want:
            where[k] = (key, start, int(kind), int(count))
    bad, big, types = 0, 0, set()
    for k, o in want.items():
        (q, j), start, kind, count = where[k]
        g = orc.gen(par[q], seed=1)
        g.set_window((win_a if q == 0 else win_b)[j])
        if start >= (1 << 17):
            d, chi = chis[q]
            g.jump_words(orc.powxmod(start, chi, d).view(np.uint32)[:351])
        else:
            g.skip(start)
        ref = np.ascontiguousarray(g.fill(kind, count))
        dt = np.uint32 if q == 0 else np.uint64
        bad += not np.array_equal(np.ascontiguousarray(o).view(dt), ref.view(dt))
        big += count > (1 << 24)
        types.add((q, kind))
    return {"requests_checked": len(want), "mismatches": int(bad), "bit_exact": bad == 0,
            "above_2^24_values": int(big),
            "types": sorted({(0, 0): "uint32", (0, 2): "float32 [0,1)", (1, 0): "uint64"}.get(
                t, str(t)) for t in types),
            "requests_in_history": len(history)}


BANK_WORKLOADS = {
    32: "bank: mtgp32_params_fast_11213[0..127], set i seeded 1234+i, one generator per set: "
        "2^21 uint32, then 2^21 float32 [0,1) per set",
    64: "bank: mtgp64dc_params_fast_11213[0..199] (the shipped 64-bit table), set i seeded "
        "5678+i, one generator per set: 2^20 uint64, then 2^20 float64 [1,2) per set"}


def run_bank(s, bits, table, nsets, seed0, n, kinds, hbm, reps=5):
    """A bank of generators, one per parameter set, each producing n values
    of each kind in turn: the plain path (pool fill, one CTA per set, like
    the reference's sample kernels) and the batched planner (autotuned;
    long requests split by jumps) on the first kind.  Device-resident
    output, CUDA-event timed, median of `reps`; the first fill of the first
    kind is kept with the windows it started from for the oracle's check."""
    import torch
    from mtgp_gb300.api import Pool, work_items
    from mtgp_gb300.params import load_table
    tbl = load_table(table)
    plist = [tbl[i] for i in range(nsets)]
    bank = Pool.create(plist, np.arange(nsets) + seed0)
    dt = torch.int32 if bits == 32 else torch.int64
    bout = torch.empty(nsets * n, dtype=dt, device="cuda")
    nbytes = nsets * n * bits // 8
    res = {"workload": BANK_WORKLOADS[bits], "bytes_per_step": nbytes}
    start = bank.windows()
    bank.fill(kinds[0][0], bout, n, stream=s)
    s.synchronize()
    first = bout.view(-1).cpu().numpy().copy()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        ts = []
        for _ in range(reps):
            ev0.record(s)
            fn()
            ev1.record(s)
            s.synchronize()
            ts.append(ev0.elapsed_time(ev1))
        return sorted(ts)[len(ts) // 2]

    for kind, name in kinds:
        bank.fill(kind, bout, n, stream=s)  # warm-up
        ms = timed(lambda: bank.fill(kind, bout, n, stream=s))
        gbs = nbytes / (ms * 1e-3) / 1e9
        res["plain " + name] = {"value": round(gbs, 2), "unit": "GB/s", "ms": round(ms, 4),
                                "pct_hbm": round(100 * gbs / hbm, 2),
                                "launch": "%d CTAs, one per set" % nsets}
    kind, name = kinds[0]
    items = work_items(np.arange(nsets), np.full(nsets, kind), np.full(nsets, n),
                       np.arange(nsets) * n * bits // 8)
    t0 = time.perf_counter()
    plan, report = bank.autotune(items, bout, stream=s, reps=3)
    setup_s = time.perf_counter() - t0
    plan.launch(bout, s)
    ms = timed(lambda: plan.launch(bout, s))
    gbs = nbytes / (ms * 1e-3) / 1e9
    res["batched " + name] = {"value": round(gbs, 2), "unit": "GB/s", "ms": round(ms, 4),
                              "pct_hbm": round(100 * gbs / hbm, 2), "plan": plan.describe(),
                              "autotune": [l for l in report.splitlines() if l.startswith("chosen")],
                              "setup_s": round(setup_s, 2)}
    res["_check"] = (bits, plist, start, n, kinds[0][0], first)
    return res


def bank_cpu(orc, bank, seconds, sample=16):
    """Oracle rate on the first `sample` sets of a bank (OpenMP over sets),
    and the GPU's first fill of those sets against it."""
    bits, plist, start, n, kind, first = bank.pop("_check")
    esz = bits // 8
    gbs, reps, nb = cpu_rate(orc, bits, plist[:sample], np.arange(sample), start[:sample],
                             np.full(sample, n), np.full(sample, kind), seconds)
    from mtgp_gb300.params import MTGP32Params, MTGP64Params, params_array
    parr = params_array(MTGP32Params if bits == 32 else MTGP64Params, plist)
    nsets = len(plist)
    win = np.ascontiguousarray(start.copy())
    ref = np.empty(nsets * n * esz, dtype=np.uint8)
    offs = (np.arange(nsets) * n * esz).astype(np.uint64)
    orc.multi_fill(bits, parr, win, np.full(nsets, n, np.uint64), np.full(nsets, kind, np.int32),
                   offs, ref, param_idx=np.arange(nsets, dtype=np.int32))
    ok = bool(np.array_equal(first.view(np.uint8), ref))
    bank["cpu_baseline"] = {"value": gbs, "unit": "GB/s", "cores": orc.max_threads(),
                            "kind": "port", "sample": "first %d sets x %d values, %d repetitions"
                                                      % (sample, n, reps)}
    bank["first_fill_bit_exact_all_sets"] = ok


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--substreams", type=int, default=N_SUB,
                    help="substreams of the batched workload (profiling runs use fewer)")
    ap.add_argument("--only", default="all",
                    choices=["all", "batched", "bank", "serve", "polys"],
                    help="profiling runs: time only one path, no e2e / plain / CPU legs")
    ap.add_argument("--serve-seconds", type=float, default=3.0,
                    help="length of each Poisson trace of the serving section")
    ap.add_argument("--serve-burst", type=int, default=100000,
                    help="requests of the burst that finds the saturation rate")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--serve-slots", type=int, default=4,
                    help="batches the server keeps in flight (measured: 4 slots "
                         "4.3-4.4 M req/s, 8 slots 4.1-4.2, 16 slots 3.9; p99 at "
                         "0.9 load 2.3-2.7 ms for each)")
    ap.add_argument("--serve-sample", type=int, default=10,
                    help="requests of each output type checked per timed serving trace")
    ap.add_argument("--uniform", type=int, default=0,
                    help="profiling runs: every substream requests this many values "
                         "(steady-state throughput instead of the lognormal workload)")
    ap.add_argument("--poly-n", type=int, default=4096,
                    help="exponents per call of the jump-polynomial section")
    ap.add_argument("--poly-reps", type=int, default=20)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--tune", action="append", default=[],
                    help="key=value tuning knob (split_chunk, batch_grid)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            dist.barrier()

    from mtgp_gb300 import build as b
    b.build()
    from mtgp_gb300.api import Pool, set_tuning, work_items
    for kv in args.tune:
        k, v = kv.split("=")
        set_tuning(k, int(v))
    from mtgp_gb300.params import jump_table, load_table

    if args.only == "polys":  # profiling run: the jump-polynomial section alone
        if rank == 0:
            print(json.dumps({"polys": run_polys(args, torch.cuda.Stream())}))
        return

    p = load_table("mtgp32_fast_11213")[0]
    nsub = args.substreams
    lens = lengths()[:nsub] if args.uniform <= 0 else np.full(nsub, args.uniform, np.int64)
    offs = np.concatenate([[0], np.cumsum(lens)[:-1]]) * 4
    total_bytes = int(lens.sum()) * 4
    s = torch.cuda.Stream()

    # --- substream setup (GPU jumps), timed separately ---
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pool = Pool.substreams(p, replica_seed(rank), nsub, jump_table(32), stream=s)
    torch.cuda.synchronize()
    jump_ms = (time.perf_counter() - t0) * 1e3
    start_windows = pool.windows()

    items = work_items(np.arange(nsub), np.zeros(nsub), lens, offs)
    out = torch.empty(total_bytes // 4, dtype=torch.int32, device="cuda")

    # --- cold: a fresh pool's substream setup, a plan with the library's
    # defaults and its first launch (the library's kernels already loaded) ---
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cpool = Pool.substreams(p, replica_seed(rank), nsub, jump_table(32), stream=s)
    s.synchronize()
    t1 = time.perf_counter()
    cplan = cpool.plan(items)
    t2 = time.perf_counter()
    cplan.launch(out, s)
    s.synchronize()
    t3 = time.perf_counter()
    cold = {"value": round(total_bytes / (t3 - t0) / 1e9, 2), "unit": "GB/s",
            "ms": round(1e3 * (t3 - t0), 2), "setup_ms": round(1e3 * (t1 - t0), 2),
            "plan_ms": round(1e3 * (t2 - t1), 2), "first_launch_ms": round(1e3 * (t3 - t2), 2),
            "what": "fresh pool: substream setup (GPU jumps) + plan (library defaults, first "
                    "use of the parameter set's jump tables) + first launch, host-timed"}
    del cplan, cpool
    # the library's autotuner picks the plan (core, split chunk, grid) on this
    # workload; the pool's windows are left as they were
    t0 = time.perf_counter()
    if args.no_autotune:
        plan, tune_report = pool.plan(items), "autotuner off"
    else:
        plan, tune_report = pool.autotune(items, out, stream=s, reps=5)
    plan_ms = (time.perf_counter() - t0) * 1e3
    plan_tasks, plan_chunk = plan.info()
    plan_cfg = plan.describe()
    # plans made later (the e2e leg) use the same configuration
    pool.set_tuning("core", plan_cfg["core"])
    pool.set_tuning("split_chunk", plan_cfg["split_chunk"] or -1)
    pool.set_tuning("batch_grid", plan_cfg["grid"])
    pool.set_tuning("jump_overlap", plan_cfg["overlap"])

    # first step, kept for the bit-exact checks
    plan.launch(out, s)
    s.synchronize()
    first_step = out.cpu().numpy().view(np.uint32).copy()
    if args.only in ("bank", "serve"):
        args.steps = 0

    # --- batched, device-resident, CUDA graph ---
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        for _ in range(args.warmup):
            plan.graph_launch(out, s)
        s.synchronize()
        barrier()
        torch.cuda.synchronize()
        ev0.record(s)
        for _ in range(args.steps):
            plan.graph_launch(out, s)
        ev1.record(s)
        s.synchronize()
        torch.cuda.synchronize()
        barrier()
    # no timed steps (the bank- and serve-only runs): no headline number
    timed = args.steps > 0
    ms = max_over_ranks(max(ev0.elapsed_time(ev1) / max(args.steps, 1), 1e-6), world)
    value = job_value(world, total_bytes, ms)
    # the last timed step's output and the windows after it, for the check
    last_step = out.cpu().numpy().view(np.uint32).copy() if args.steps else None
    end_windows = pool.windows()
    nlaunched = 1 + args.warmup + args.steps
    # the persistent kernel (+ the staged-window copy of split plans) per
    # step; the work-counter reset is a memset, not a kernel
    launches = plan_cfg["kernels_per_launch"] * args.steps

    if args.only != "all":
        args.plain_steps = 0
        args.no_cpu = True
    # --- e2e: host items in, host output back, every step.  Each step refills
    # a plan from the host items (pool_replan: planned on the host, uploaded
    # with the launch) and copies its whole output to pinned host memory;
    # two plans and output buffers let step k's copy overlap step k+1's
    # planning and generation.  Every copy is inside the timed region. ---
    e2e_steps = 0 if args.only != "all" else max(3, min(args.steps, 10))
    nbuf = 2 if e2e_steps else 0
    outs = [out, torch.empty_like(out)][:nbuf]
    host_out = [torch.empty(total_bytes // 4, dtype=torch.int32, pin_memory=True)
                for _ in range(nbuf)]
    plans = [pool.plan(items) for _ in range(nbuf)]
    cstream = torch.cuda.Stream()
    gen_done = [torch.cuda.Event() for _ in range(nbuf)]
    copy_done = [torch.cuda.Event() for _ in range(nbuf)]
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        b = k % 2
        if k >= 2:
            copy_done[b].synchronize()   # buffer and plan of step k-2 are free
        pool.replan(items, plans[b])
        plans[b].launch(outs[b], s)
        gen_done[b].record(s)
        cstream.wait_event(gen_done[b])
        with torch.cuda.stream(cstream):
            host_out[b].copy_(outs[b], non_blocking=True)
        copy_done[b].record(cstream)
    cstream.synchronize()
    s.synchronize()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / max(e2e_steps, 1), world)
    e2e = job_value(world, total_bytes, e2e_s * 1e3)
    del outs, host_out, plans
    # the plain and bank legs run on the default generation core, not on the
    # batched plan's
    pool.set_tuning("core", 2)

    # --- plain: one launch (one CTA) per substream ---
    plain_ms = None
    if args.plain_steps > 0:
        torch.cuda.synchronize()
        ev0.record(s)
        for _ in range(args.plain_steps):
            for j in range(nsub):
                pool.fill_stream(j, 0, out, int(lens[j]), stream=s, byte_offset=int(offs[j]))
        ev1.record(s)
        s.synchronize()
        plain_ms = ev0.elapsed_time(ev1) / args.plain_steps
    # the same launches spread over 32 CUDA streams, from a CUDA graph
    plain_conc_ms = None
    if args.plain_steps > 0:
        plain_conc_ms = plain_concurrent(pool, lens, offs, out, nstreams=32,
                                         steps=max(args.plain_steps, 3))

    # --- banks: one CTA per parameter set (the reference sample's launch
    # shape), then the same work through the batched planner ---
    hbm, peak_kind = peaks()
    banks = {}
    if args.only in ("all", "bank"):
        banks["bank32"] = run_bank(s, 32, "mtgp32_fast_11213", 128, 1234, 1 << 21,
                                   ((0, "uint32"), (2, "float32 [0,1)")), hbm)
        banks["bank64"] = run_bank(s, 64, "mtgp64dc_fast_11213", 200, 5678, 1 << 20,
                                   ((0, "uint64"), (1, "float64 [1,2)")), hbm)

    # --- jump polynomials for arbitrary offsets, on the GPU ---
    polys, single = None, None
    if rank == 0 and args.only == "all":
        polys = run_polys(args, s)
        single = run_single(s)

    # --- serving: continuous batching over resident streams ---
    serve, serve_chk = None, None
    if rank == 0 and not args.no_serve and args.only in ("all", "serve"):
        serve, serve_chk = run_serving(args, s, local)

    # --- store-only HBM bandwidth, beside the copy peak of the roofline ---
    wpeak = write_peak() if rank == 0 and args.only == "all" else None

    state_bytes = 2 * nsub * 351 * 4
    achieved = (total_bytes + state_bytes) / (ms * 1e-3) / 1e9
    chosen = [l for l in tune_report.splitlines() if l.startswith("chosen:")]
    kernel = (chosen[0][len("chosen:"):].split(", chunk=")[0].strip() if chosen else
              "k_batch32xk<%d>%s" % (plan_cfg["core"], " after k_jump_part5 (%d windows jumped "
                                     "ahead)" % plan_cfg["prejumps"] if plan_cfg["prejumps"] else ""))
    # DRAM bytes (read + write) per step of the plan's kernels, from an ncu
    # capture of the same plan on the same workload (profiles/); reported
    # only when the autotuner chose the captured plan
    plan_key = (plan_cfg["core"], plan_cfg["split_chunk"], plan_cfg["grid"], plan_cfg["prejumps"])
    cap = CAPTURED_TRAFFIC.get(plan_key) if (nsub == N_SUB and args.uniform <= 0) else None
    roofline = {"bound": "hbm", "achieved": round(achieved, 1) if timed else None,
                "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 4) if timed else None, "peak_kind": peak_kind,
                "traffic": cap["bytes"] if cap else None,
                "traffic_source": cap["source"] if cap else "no capture of this plan",
                "algorithmic_bytes": total_bytes + state_bytes, "kernel": kernel}

    cpu, check = None, None
    if rank == 0 and not args.no_cpu:
        from oracle.bind import Oracle, build as obuild
        obuild()
        orc = Oracle()
        cpu_gbs, reps, words, ok = cpu_baseline(orc, p, start_windows, lens, 256, first_step,
                                                args.cpu_seconds)
        cpu = {"value": round(cpu_gbs, 3), "unit": "GB/s", "cores": orc.max_threads(),
               "kind": "port",
               "sample": "first 256 substreams of the workload (%d uint32), %d repetitions"
                         % (words, reps),
               "gpu_first_step_bit_exact": ok}
        if last_step is not None:
            check = full_check(orc, p, start_windows, lens, first_step, last_step, end_windows,
                               nlaunched)
        for bk in banks.values():
            bank_cpu(orc, bk, min(args.cpu_seconds, 3.0))
        if serve_chk is not None:
            serve["check"] = serve_check(orc, serve_chk)
        if polys is not None:
            polys["cpu_baseline"] = poly_cpu_baseline(orc, min(args.cpu_seconds, 5.0))

    for bk in banks.values():
        bk.pop("_check", None)
    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 2) if timed else None, "unit": "GB/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 4) if timed else None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": WORKLOAD,
                       "output_bytes_per_step": total_bytes,
                       "l2": "no flush: each step writes %.2f GB, > 129 MB L2" % (total_bytes / 1e9),
                       "parallelism": "replicas" if world > 1 else "single"},
            "pct_hbm": round(100 * value / world / hbm, 2) if timed else None,
            "plain": None if plain_ms is None else {
                "value": round(world * total_bytes / (plain_ms * 1e-3) / 1e9, 3), "unit": "GB/s",
                "ms_per_step": round(plain_ms, 2), "launches_per_step": nsub},
            "plain_concurrent": None if plain_conc_ms is None else {
                "value": round(world * total_bytes / (plain_conc_ms * 1e-3) / 1e9, 3),
                "unit": "GB/s", "ms_per_step": round(plain_conc_ms, 3),
                "launches_per_step": nsub,
                "how": "one CTA per substream, launches dealt to 32 CUDA streams, replayed "
                       "from one CUDA graph"},
            "batched_over_plain": None if plain_ms is None or not timed else round(plain_ms / ms, 2),
            "batched_over_plain_concurrent": None if plain_conc_ms is None or not timed
            else round(plain_conc_ms / ms, 2),
            "write_peak": None if wpeak is None else {
                "value": wpeak, "unit": "GB/s",
                "how": "4 GiB written by one torch fill kernel, best of 10",
                "pct_of_write_peak": round(100 * value / world / wpeak, 2) if timed else None},
            "check": check,
            "cold": cold,
            "banks": banks or None,
            "single": single,
            "jump_setup": {"ms": round(jump_ms, 2), "us_per_substream": round(1e3 * jump_ms / nsub, 2)},
            "plan": {"tasks": plan_tasks, "split_chunk": plan_chunk, "config": plan_cfg,
                     "autotune_ms": round(plan_ms, 1),
                     "autotune": [l for l in tune_report.strip().splitlines()]},
            "serve": serve,
            "jump_polys": polys,
            "e2e": None if not e2e_steps else {
                "value": round(e2e, 3), "unit": "GB/s", "h2d_bytes_per_step": 32 * nsub,
                "d2h_bytes_per_step": total_bytes},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "gpu_launches": launches,
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
