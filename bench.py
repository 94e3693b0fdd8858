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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--substreams", type=int, default=N_SUB,
                    help="substreams of the batched workload (profiling runs use fewer)")
    ap.add_argument("--only", default="all", choices=["all", "batched", "bank"],
                    help="profiling runs: time only one path, no e2e / plain / CPU legs")
    ap.add_argument("--uniform", type=int, default=0,
                    help="profiling runs: every substream requests this many values "
                         "(steady-state throughput instead of the lognormal workload)")
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

    p = load_table("mtgp32_fast_11213")[0]
    nsub = args.substreams
    lens = lengths()[:nsub] if args.uniform <= 0 else np.full(nsub, args.uniform, np.int64)
    offs = np.concatenate([[0], np.cumsum(lens)[:-1]]) * 4
    total_bytes = int(lens.sum()) * 4
    s = torch.cuda.Stream()

    # --- substream setup (GPU jumps), timed separately ---
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pool = Pool.substreams(p, SEED + rank, nsub, jump_table(32), stream=s)
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
        plan, tune_report = pool.autotune(items, out, stream=s, reps=2)
    plan_ms = (time.perf_counter() - t0) * 1e3
    plan_tasks, plan_chunk = plan.info()

    # first step, kept for the CPU-baseline leg's bit-exact check
    plan.launch(out, s)
    s.synchronize()
    first_step = out[:int(lens[:256].sum())].cpu().numpy().view(np.uint32).copy()
    if args.only == "bank":
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
    ms = max(ev0.elapsed_time(ev1) / max(args.steps, 1), 1e-6)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * total_bytes / (ms * 1e-3) / 1e9
    launches = 2 * args.steps  # memset of the work counter + the persistent kernel

    if args.only != "all":
        args.plain_steps = 0
        args.no_cpu = True
    # --- e2e: host items in, host output back, every step ---
    e2e_steps = 0 if args.only != "all" else max(3, min(args.steps, 10))
    host_out = torch.empty(total_bytes // 4, dtype=torch.int32, pin_memory=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        with torch.cuda.stream(s):
            pool.submit(items, out, s)
            host_out.copy_(out, non_blocking=True)
        s.synchronize()
    e2e_s = (time.perf_counter() - t0) / max(e2e_steps, 1)
    e2e = world * total_bytes / e2e_s / 1e9

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
    bank_reps = 0 if args.only == "batched" else 5
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

    hbm, peak_kind = peaks()
    state_bytes = 2 * nsub * 351 * 4
    achieved = (total_bytes + state_bytes) / (ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 4), "peak_kind": peak_kind,
                "traffic": None, "kernel": "k_batch32<351,256,1024>"}

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
            "bank": {"value": round(bank_gbs, 2), "unit": "GB/s", "ms": round(bank_ms, 3),
                     "workload": "128 sets x 2^21 uint32, seeds 1234+i, one CTA per set"},
            "jump_setup": {"ms": round(jump_ms, 2), "us_per_substream": round(1e3 * jump_ms / nsub, 2)},
            "plan": {"tasks": plan_tasks, "split_chunk": plan_chunk,
                     "autotune_ms": round(plan_ms, 1),
                     "autotune": [l for l in tune_report.strip().splitlines()]},
            "e2e": {"value": round(e2e, 3), "unit": "GB/s", "h2d_bytes_per_step": 24 * nsub,
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
