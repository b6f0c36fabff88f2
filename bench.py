"""Benchmark of the GB300 Legendre<->Chebyshev transform.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload single] [--N 1048576] [--maxs 64] [--no-cpu-baseline]

Workload (default): one vector of N = 2^20 Legendre coefficients
c_n = s_n/(n+1), s_n = +-1 iid (seeded), maxs = 64 (s = 64, L = 12), plain
FP64.  One step = one L2C and one C2L of that vector; the metric counts the
coefficients transformed (2 N per step) per second.

  value   device-resident: inputs already in HBM, plan built, outputs zeroed
          before each step; L2 flushed (256 MiB write) between steps; CUDA
          events on the plan's stream around each step.
  e2e     the same through execute() with host (pinned) buffers: host->device
          copies of input and output (execute accumulates into its output, as
          the reference), kernels, device->host copy of the result, per step.
  roofline  dominant kernel (by time) timed live with per-phase CUDA events;
          FP64 work in the reference's own flop count; peak = FP64 DGEMM
          throughput measured in this run (cuBLAS, float64 matmul).
  cpu_baseline  the oracle port of the reference algorithm (OpenMP, all host
          cores) on the same vector, rank 0 only, ~10 s bounded sample.

--impl reference: the reference's CPU algorithm (the oracle port; the
reference sources are not available on the GPU machine) on all host cores,
same workload, same metric.
Under torchrun each rank runs the same workload on its own GPU (independent
replicas, weak scaling); value = all coefficients / max time over ranks.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "legendre-to-chebyshev_gb300")
METRIC = "L2C/C2L coeffs/sec at ≤1e-14 rel err vs FP64 oracle; mixed vs plain FP64"


def sign_decay_input(N, seed):
    rng = np.random.default_rng(seed)
    return rng.choice([-1.0, 1.0], N) / (np.arange(N, dtype=np.float64) + 1.0)


def near_flops(N, s, direction):
    """Reference flop count of the near-field band (directM / directL)."""
    h = 2 * s
    nL = N // h
    i0 = (nL - 1) * h
    band = sum(3 * (h if n < h else 2 * h - n) for n in range(0 if direction == 0 else 2, 4 * s, 2))
    f = (nL - 1) * band
    if direction == 0:
        n = 0
        while 2 * n + i0 < N:
            f += 3 * (N - (2 * n + i0))
            n += 1
        return f + N
    f += 3 * N
    for n in range(1, N - i0):
        f += 3 * (N - (2 * n + i0))  # may be negative: the reference wraps; the sum stays right
    return f + 2 * N


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_fp64_peak(torch, dev):
    """FP64 DGEMM throughput (TFLOP/s), best of 5, cuBLAS float64 matmul."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    return best


def cpu_run(N, maxs, u, seconds, threads):
    """Oracle port: L2C + C2L of u repeatedly for about `seconds`; returns
    (coefficients per second, outputs, reps)."""
    sys.path.insert(0, REPO)
    from oracle import oracle

    oracle.set_threads(threads)
    o = oracle.Oracle(N, maxs, 2)
    outs = [np.zeros(N), np.zeros(N)]
    times = []
    t_start = time.perf_counter()
    while True:
        for d in (0, 1):
            outs[d][:] = 0
        t0 = time.perf_counter()
        o.execute(u, outs[0], 0)
        o.execute(u, outs[1], 1)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start > seconds and len(times) >= 2:
            break
    return 2 * N / statistics.median(times), outs, len(times)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    N, maxs = args.N, args.maxs
    u = sign_decay_input(N, 1)
    threads = os.cpu_count() or 1
    sys.path.insert(0, REPO)
    from oracle import oracle

    oracle.set_threads(threads)
    o = oracle.Oracle(N, maxs, 2)
    outs = [np.zeros(N), np.zeros(N)]
    for _ in range(args.warmup):
        o.execute(u, outs[0], 0)
        o.execute(u, outs[1], 1)
    times = []
    for _ in range(args.steps):
        outs[0][:] = 0
        outs[1][:] = 0
        t0 = time.perf_counter()
        o.execute(u, outs[0], 0)
        o.execute(u, outs[1], 1)
        times.append(time.perf_counter() - t0)
    t = sum(times) / len(times)
    value = 2 * N / t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "coef/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(N, maxs),
        "cpu_baseline": {"value": value, "unit": "coef/s", "cores": threads, "kind": "port",
                         "sample": f"full workload: L2C + C2L of one N={N} vector per step, "
                                   f"{args.steps} steps; oracle port of the reference algorithm "
                                   "(its sources are not on this machine)"},
        "e2e": {"value": value, "unit": "coef/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def workload_config(N, maxs):
    sys.path.insert(0, PKG)
    L = math.ceil(math.log2(N / maxs)) - 2
    s = math.ceil(N / 2 ** (L + 2)) if L >= 1 else 0
    return {"workload": f"single vector L2C + C2L, N={N}, maxs={maxs} (s={s}, L={L}), "
                        "c_n = s_n/(n+1), plain FP64",
            "N": N, "maxs": maxs, "s": s, "L": L, "precision": "fp64",
            "l2_flush": "256 MiB write between steps", "vectors_per_step": 2}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="single", choices=["single"])
    ap.add_argument("--N", type=int, default=1 << 20)
    ap.add_argument("--maxs", type=int, default=64)
    ap.add_argument("--precompute", type=int, default=0,
                    help="1: keep the near-field band weights in device memory (create_fmm's "
                         "precompute argument)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    sys.path.insert(0, PKG)
    import importlib.util

    spec = importlib.util.spec_from_file_location("l2c_pkg_build", os.path.join(PKG, "build.py"))
    bmod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bmod)
    if rank == 0:
        bmod.build()
    barrier()
    import l2c_gb300 as l2c

    abi = l2c.cuda_abi()
    N, maxs = args.N, args.maxs
    u = sign_decay_input(N, 1 + rank)
    plan = l2c.Plan(N, maxs, precompute=args.precompute)
    stream = torch.cuda.ExternalStream(plan.stream, device=dev)
    du = torch.from_numpy(u).to(dev)
    douts = [torch.zeros(N, dtype=torch.float64, device=dev) for _ in range(2)]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    peak = measured_fp64_peak(torch, dev)

    def step():
        with torch.cuda.stream(stream):
            flush.fill_(1)
            douts[0].zero_()
            douts[1].zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.execute_async(du, douts[0], 0)
        plan.execute_async(du, douts[1], 1)
        e1.record(stream)
        return e0, e1

    for _ in range(args.warmup):
        step()
    plan.synchronize()
    torch.cuda.synchronize()

    # ---- timed region (device resident) ----
    abi.l2c_gpu_profile(plan._gpu, 1)
    launches0 = abi.l2c_gpu_launch_count(plan._gpu)
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    t_wall0 = time.perf_counter()
    evs = [step() for _ in range(args.steps)]
    plan.synchronize()
    torch.cuda.synchronize()
    barrier()
    t_wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    launches = abi.l2c_gpu_launch_count(plan._gpu) - launches0
    ms = [a.elapsed_time(b) for a, b in evs]
    ms_step = sum(ms) / len(ms)
    import ctypes

    pms = (ctypes.c_double * 8)()
    pl = (ctypes.c_size_t * 8)()
    abi.l2c_gpu_profile_read(plan._gpu, pms, pl)
    abi.l2c_gpu_profile(plan._gpu, 0)
    names = ["gather", "near", "leaf_up", "tree_up", "far", "tree_down", "leaf_down", "direct"]
    phases = {names[i]: {"ms_per_step": pms[i] / args.steps, "launches_per_step": pl[i] / args.steps}
              for i in range(8) if pl[i]}
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([ms_step], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
    value = 2 * N * world / (ms_step * 1e-3)

    # ---- e2e through execute() with pinned host buffers ----
    hin = torch.from_numpy(u).pin_memory()
    houts = [torch.zeros(N, dtype=torch.float64).pin_memory() for _ in range(2)]
    e2e_t = []
    for it in range(args.warmup + args.steps):
        for h in houts:
            h.zero_()
        t0 = time.perf_counter()
        plan.execute(hin, houts[0], 0)
        plan.execute(hin, houts[1], 1)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            e2e_t.append(dt)
    e2e_step = sum(e2e_t) / len(e2e_t)
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([e2e_step], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_step = float(t.item())
    e2e_value = 2 * N * world / e2e_step

    # ---- roofline of the dominant kernel ----
    dom = max(phases, key=lambda k: phases[k]["ms_per_step"])
    L, s, _ = l2c.geometry(N, maxs)
    roof = None
    if dom == "near":
        flops_per_launch = (near_flops(N, s, 0) + near_flops(N, s, 1)) / 2.0
        avg_ms = phases["near"]["ms_per_step"] / phases["near"]["launches_per_step"]
        achieved = flops_per_launch / (avg_ms * 1e-3) / 1e12
        roof = {"bound": "tensor", "pipe": "fp64", "kernel": "k_near (near-field band)",
                "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": None,
                "peak_source": "FP64 DGEMM measured in this run (cuBLAS float64 matmul 4096^3)",
                "flops_per_launch": flops_per_launch, "avg_launch_ms": avg_ms}
    total_flops = plan.flops(0) + plan.flops(1)

    line = {
        "metric": METRIC, "value": value, "unit": "coef/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded c_n = s_n/(n+1))",
        "config": dict(workload_config(N, maxs), precompute=args.precompute),
        "e2e": {"value": e2e_value, "unit": "coef/s", "h2d_bytes_per_step": 2 * 16 * N,
                "d2h_bytes_per_step": 2 * 8 * N, "ms_per_step": e2e_step * 1e3},
        "gpu_launches": int(launches),
        "clocks": clk,
        "roofline": roof,
        "phases": phases,
        "fp64_tflops_whole_step": total_flops / (ms_step * 1e-3) / 1e12,
        "wall_s_timed_region": t_wall,
        "plan": {"L": L, "s": s, "Nb": plan.Nb},
    }

    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        cpu_value, outs, reps = cpu_run(N, maxs, u, args.cpu_seconds, threads)
        line["cpu_baseline"] = {
            "value": cpu_value, "unit": "coef/s", "cores": threads, "kind": "port",
            "sample": f"{reps} repetitions of the full step (L2C + C2L, N={N}), median; "
                      "oracle port of the reference algorithm with OpenMP"}
        got = [douts[0].cpu().numpy(), douts[1].cpu().numpy()]
        line["max_rel_err_vs_oracle"] = {
            "l2c": float(np.max(np.abs(got[0] - outs[0])) / np.max(np.abs(outs[0]))),
            "c2l": float(np.max(np.abs(got[1] - outs[1])) / np.max(np.abs(outs[1])))}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
