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
    """Serving section: a check trace whose responses are kept for the
    oracle, a burst that finds the saturation rate, then Poisson traces at
    0.3 / 0.6 / 0.9 of it with p50 / p99 latency (submission to the result
    resident in device memory)."""
    import torch
    from mtgp_gb300.api import Pool, Server, requests, set_tuning
    from mtgp_gb300.params import jump_table, load_table
    # the library's default planning (the batched section's tuning is global)
    set_tuning("core", 2)
    set_tuning("split_chunk", 0)
    set_tuning("batch_grid", 0)
    p32 = load_table("mtgp32_fast_11213")[0]
    p64 = load_table("mtgp64dc_fast_11213")[0]
    a = Pool.substreams(p32, SEED, 4096, jump_table(32), stream=s)
    b = Pool.substreams(p64, SEED, 256, jump_table(64), stream=s)
    s.synchronize()
    win_a, win_b = a.windows(), b.windows()
    srv = Server(a, b, budget_bytes=8 << 30, slots=args.serve_slots, max_batch=8192)
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
    check = (pool, stream, kind, count, skip, [o.cpu().numpy() for o in outs], win_a, win_b)
    del outs

    def run(tr, arrivals):
        c0, b0, k0 = srv.stats()
        wall = srv.replay(requests(*tr), arrivals)
        c1, b1, k1 = srv.stats()
        lat, st = srv.results()
        assert (st[c0:c1] == 0).all(), "failed requests"
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
        wall, nbytes, batches, lat = run(serve_trace(rng, n), np.zeros(n))
        sat = n / wall
        out["saturation"] = {"requests": n, "req_per_s": round(sat, 1),
                             "GB_per_s": round(nbytes / wall / 1e9, 2), "batches": batches}
        rates = []
        for load in (0.3, 0.6, 0.9):
            rate = load * sat
            n = max(200, int(rate * args.serve_seconds))
            arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
            wall, nbytes, batches, lat = run(serve_trace(rng, n), arrivals)
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
    return out, check


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


def serve_check(orc, chk):
    """Every response of the check trace against the oracle: each stream
    replayed in submission order from the windows the pools started from
    (offsets of 2^17 or more by X^offset mod chi, as the server does)."""
    from mtgp_gb300.params import load_table
    pool, stream, kind, count, skip, outs, win_a, win_b = chk
    par = {0: load_table("mtgp32_fast_11213")[0], 1: load_table("mtgp64dc_fast_11213")[0]}
    chis = {}
    for q, p in par.items():
        seq = orc.gen(p, seed=1).fill(0, 2 * p.mexp)
        chis[q] = orc.minpoly((seq & 1).astype(np.uint8))
    gens, bad = {}, 0
    for k in range(len(pool)):
        q, j = int(pool[k]), int(stream[k])
        if (q, j) not in gens:
            o = orc.gen(par[q], seed=1)
            o.set_window((win_a if q == 0 else win_b)[j])
            gens[(q, j)] = o
        o = gens[(q, j)]
        if int(skip[k]) >= (1 << 17):
            d, chi = chis[q]
            o.jump_words(orc.powxmod(int(skip[k]), chi, d).view(np.uint32)[:351])
        else:
            o.skip(int(skip[k]))
        ref = np.ascontiguousarray(o.fill(int(kind[k]), int(count[k])))
        dt = np.uint32 if q == 0 else np.uint64
        bad += not np.array_equal(outs[k].view(dt), ref.view(dt))
    return {"requests": len(pool), "mismatches": int(bad), "bit_exact": bad == 0,
            "jumped": int((skip >= (1 << 17)).sum())}


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
    ap.add_argument("--serve-slots", type=int, default=8,
                    help="batches the server keeps in flight (CUDA streams)")
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
    set_tuning("core", plan_cfg["core"])
    set_tuning("split_chunk", plan_cfg["split_chunk"] or -1)
    set_tuning("batch_grid", plan_cfg["grid"])

    # first step, kept for the CPU-baseline leg's bit-exact check
    plan.launch(out, s)
    s.synchronize()
    first_step = out[:int(lens[:256].sum())].cpu().numpy().view(np.uint32).copy()
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
    ms = max_over_ranks(max(ev0.elapsed_time(ev1) / max(args.steps, 1), 1e-6), world)
    value = job_value(world, total_bytes, ms)
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
    # the plain and bank legs run on the default generation core, not on the
    # batched plan's
    set_tuning("core", 2)

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

    # --- bank: 128 parameter sets, 2^21 uint32 each, one CTA per set ---
    bank_reps = 0 if args.only in ("batched", "serve") else 5
    tbl = load_table("mtgp32_fast_11213")
    bank = Pool.create([tbl[i] for i in range(128)], np.arange(128) + 1234)
    nb = 1 << 21
    bout = torch.empty(128 * nb, dtype=torch.int32, device="cuda")
    for _ in range(2):
        bank.fill(0, bout, nb, stream=s)
    s.synchronize()
    ev0.record(s)
    for _ in range(bank_reps):
        bank.fill(0, bout, nb, stream=s)
    ev1.record(s)
    s.synchronize()
    bank_ms = max(ev0.elapsed_time(ev1) / max(bank_reps, 1), 1e-6)
    bank_gbs = 128 * nb * 4 / (bank_ms * 1e-3) / 1e9
    # the same bank through the batched planner: each set's 2^21 values split
    # into chunks that start with in-kernel jumps (autotuned; the first plan
    # computes 128 characteristic and jump polynomials, outside the timing)
    bank_b = None
    if bank_reps:
        bitems = work_items(np.arange(128), np.zeros(128), np.full(128, nb),
                            np.arange(128) * nb * 4)
        t0 = time.perf_counter()
        bplan, _ = bank.autotune(bitems, bout, stream=s, reps=3)
        setup_s = time.perf_counter() - t0
        for _ in range(3):
            bplan.launch(bout, s)
        s.synchronize()
        ev0.record(s)
        for _ in range(bank_reps):
            bplan.launch(bout, s)
        ev1.record(s)
        s.synchronize()
        bb_ms = max(ev0.elapsed_time(ev1) / bank_reps, 1e-6)
        bank_b = {"value": round(128 * nb * 4 / (bb_ms * 1e-3) / 1e9, 2), "unit": "GB/s",
                  "ms": round(bb_ms, 3), "plan": bplan.describe(),
                  "setup_s": round(setup_s, 2)}

    # --- jump polynomials for arbitrary offsets, on the GPU ---
    polys, single = None, None
    if rank == 0 and args.only == "all":
        polys = run_polys(args, s)
        single = run_single(s)

    # --- serving: continuous batching over resident streams ---
    serve, serve_chk = None, None
    if rank == 0 and not args.no_serve and args.only in ("all", "serve"):
        serve, serve_chk = run_serving(args, s, local)

    hbm, peak_kind = peaks()
    state_bytes = 2 * nsub * 351 * 4
    achieved = (total_bytes + state_bytes) / (ms * 1e-3) / 1e9
    chosen = [l for l in tune_report.splitlines() if l.startswith("chosen:")]
    kernel = chosen[0][len("chosen:"):].split(", chunk=")[0].strip() if chosen else None
    # DRAM bytes (read + write) of one launch of the batched kernel on this
    # workload, measured once with ncu (dram__bytes_read.sum +
    # dram__bytes_write.sum = 11.58 MB + 1.69 GB); only valid for the full
    # default workload
    traffic = 1.70e9 if (nsub == N_SUB and args.uniform <= 0) else None
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 4), "peak_kind": peak_kind,
                "traffic": traffic, "algorithmic_bytes": total_bytes + state_bytes,
                "kernel": kernel}

    cpu = None
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
        if serve_chk is not None:
            serve["check"] = serve_check(orc, serve_chk)
        if polys is not None:
            polys["cpu_baseline"] = poly_cpu_baseline(orc, min(args.cpu_seconds, 5.0))

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": "GB/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": WORKLOAD,
                       "output_bytes_per_step": total_bytes,
                       "l2": "no flush: each step writes %.2f GB, > 129 MB L2" % (total_bytes / 1e9),
                       "parallelism": "replicas" if world > 1 else "single"},
            "pct_hbm": round(100 * value / world / hbm, 2),
            "plain": None if plain_ms is None else {
                "value": round(world * total_bytes / (plain_ms * 1e-3) / 1e9, 3), "unit": "GB/s",
                "ms_per_step": round(plain_ms, 2), "launches_per_step": nsub},
            "batched_over_plain": None if plain_ms is None else round(plain_ms / ms, 2),
            "bank_batched": bank_b,
            "bank": None if not bank_reps else {
                "value": round(bank_gbs, 2), "unit": "GB/s", "ms": round(bank_ms, 3),
                "workload": "128 sets x 2^21 uint32, seeds 1234+i, one CTA per set"},
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
