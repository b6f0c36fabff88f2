"""Benchmark of the GB300 Legendre<->Chebyshev transform.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload single] [--N 1048576] [--maxs 64] [--no-cpu-baseline]

Workload (default): one vector of N = 2^20 Legendre coefficients
c_n = s_n/(n+1), s_n = +-1 iid (seeded), maxs = 64 (s = 64, L = 12), plain
FP64.  One step = one L2C and one C2L of that vector; the metric counts the
coefficients transformed (2 N per step) per second.

  value   device-resident: inputs already in HBM, plan built, outputs zeroed
          before each step; L2 flushed (256 MiB write) between steps; CUDA
          events on the plan's stream around each step; each call replays the
          CUDA graph the library captured for its shape (as any repeated call).
  e2e     the same through execute() with host (pinned) buffers: host->device
          copies of input and output (execute accumulates into its output, as
          the reference), kernels, device->host copy of the result, per step.
  roofline  dominant kernel (by time) timed live with per-phase CUDA events in
          a second pass of the same K steps (direct launches, no graph);
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


def gauss2_lines(count, N, seed):
    """Lines of a 64x64x1024-style array: iid N(0,1) times (n+1)^-2 along the line."""
    rng = np.random.default_rng(seed)
    return rng.standard_normal((count, N)) / (np.arange(N, dtype=np.float64) + 1.0) ** 2


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


def hbm_peak_gbs():
    """Measured copy bandwidth (MEASURED_PEAKS.json), else the 6.8 TB/s fallback."""
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            v = json.load(f).get("hbm_gbs")
        if v:
            return float(v), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, ValueError):
        pass
    return 6800.0, "fallback 6.8 TB/s"


FP64_PEAK_SOURCE = ("FP64 DGEMM measured in this run (cuBLAS float64 matmul 4096^3); "
                    "MEASURED_PEAKS.json holds no FP64 figure")
BAND_PROFILE = "profiles/band_single_N1048576.md"


def profile_traffic(rel_path, calls=None):
    """DRAM bytes from a committed ncu summary: dram__bytes_read.sum +
    dram__bytes_write.sum over the summary's launch columns ("|
    dram__bytes_read.sum | 25.2 MB | 25.2 MB |"), per launch (their mean) or,
    with calls, per call (their sum over the calls the columns cover)."""
    units = {"B": 1.0, "KB": 1e3, "MB": 1e6, "GB": 1e9}
    try:
        with open(os.path.join(REPO, rel_path)) as f:
            rows = [ln for ln in f if ln.startswith("| dram__bytes_")]
    except OSError:
        return None
    cols = None
    for ln in rows:
        name = ln.split("|")[1].strip()
        if name not in ("dram__bytes_read.sum", "dram__bytes_write.sum"):
            continue
        vals = []
        for cell in ln.strip().strip("|").split("|")[1:]:
            parts = cell.split()
            vals.append(float(parts[0]) * units[parts[1] if len(parts) > 1 else "B"])
        cols = vals if cols is None else [a + b for a, b in zip(cols, vals)]
    if not cols:
        return None
    return sum(cols) / (calls if calls else len(cols))


def phase_roofline(wl, L, s, Nb, phases, fp64_tf, hbm_gbs, lagrange):
    """Per FMM step of one bench step (both calls): the reference's flop count
    and the algorithmic DRAM bytes of that step, over its CUDA-event time, as
    fractions of the measured FP64 DGEMM rate and HBM copy bandwidth."""
    N, count, M = wl.N, wl.count, 18
    MM, K = M * M, 2 * ((2 << (L - 1)) - 1)
    slots = 2 * Nb
    calls = len(wl.calls)
    c2l_calls = sum(1 for d, _, _ in wl.calls if d == 1)
    tr = 4 if lagrange else 1
    up = sum(((2 << l) - 2) * MM * tr for l in range(1, L))
    down = sum(((2 << (l + 1)) - 2) * MM * tr for l in range(0, L - 1))
    col = 2 * slots * M * 8  # one pass over a vector's tree (both parities)
    work = {  # name: (flops, bytes) per bench step
        "gather": (c2l_calls * count * N, c2l_calls * count * 16 * N),
        "near": (sum(near_flops(N, s, d) for d, _, _ in wl.calls) * count,
                 calls * count * 24 * N),
        "leaf_up": (calls * count * 2 * 2 * K * s * M, calls * count * (8 * N + 2 * K * M * 8)),
        "tree_up": (calls * count * 2 * up, calls * count * 2 * col),
        "far": (calls * count * 2 * 3 * Nb * 2 * MM,
                calls * (3 * Nb * MM * 8 + count * 2 * col)),
        "tree_down": (calls * count * 2 * down, calls * count * 2 * col),
        "leaf_down": (calls * count * 2 * 2 * K * s * M,
                      calls * count * (2 * K * M * 8 + 16 * N)),
    }
    out = {}
    for name, (fl, by) in work.items():
        if name not in phases or phases[name]["ms_per_step"] <= 0:
            continue
        t = phases[name]["ms_per_step"] * 1e-3
        out[name] = {"ms_per_step": round(t * 1e3, 4),
                     "fp64_tflops": round(fl / t / 1e12, 4),
                     "frac_fp64": round(fl / t / 1e12 / fp64_tf, 3),
                     "alg_gbs": round(by / t / 1e9, 1),
                     "frac_hbm": round(by / t / 1e9 / hbm_gbs, 3)}
    return out


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


def rank_env():
    """(rank, world size, local rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class Ranks:
    """Barrier and max-over-ranks for the timed region; one process per GPU.
    Every rank runs the same workload on its own device (independent replicas,
    no data-path collective), so the whole-job value is the coefficients of all
    ranks over the slowest rank's time (aggregate_value)."""

    def __init__(self, world, backend, device):
        self.world, self.device = world, device
        if world > 1:
            import torch.distributed as dist

            if backend == "nccl":
                dist.init_process_group("nccl", device_id=device)
            else:
                dist.init_process_group(backend)

    def barrier(self):
        if self.world > 1:
            import torch.distributed as dist

            dist.barrier()

    def max(self, x):
        if self.world == 1:
            return x
        import torch
        import torch.distributed as dist

        t = torch.tensor([x], device=self.device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())


def aggregate_value(coefs_per_step_per_rank, world, ms_max):
    """Whole-job coefficients per second: every rank's coefficients over the max time."""
    return coefs_per_step_per_rank * world / (ms_max * 1e-3)


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


def ragged_lengths(count, seed, lo=64, hi=65536):
    """N log-uniform in [lo, hi], seeded."""
    rng = np.random.default_rng(seed)
    return np.round(np.exp(rng.uniform(np.log(lo), np.log(hi), count))).astype(np.int64)


def workload_config(N, maxs, workload="single", count=1, total=None, lagrange=0):
    if workload == "ragged":
        return {"workload": f"ragged list: {count} vectors, N log-uniform in [64, 65536] (seeded), "
                            f"{total} coefficients in total, iid U[-1,1]; L2C and C2L, "
                            f"maxs={maxs}, plain FP64, one set of launches per direction",
                "vectors": count, "total_coefficients": total, "maxs": maxs,
                "precision": "fp64", "l2_flush": "256 MiB write between steps",
                "transforms_per_step": 2 * count}
    L = math.ceil(math.log2(N / maxs)) - 2
    s = math.ceil(N / 2 ** (L + 2)) if L >= 1 else 0
    form = "nodal (lagrange=1)" if lagrange else "plain FP64"
    if workload == "batch":
        desc = (f"batched lines: {count} transforms of N={N} along the last axis of a "
                f"64x64x{N} float64 array (dist={N}, stride=1), x = N(0,1)(n+1)^-2; "
                f"L2C then C2L of the result, maxs={maxs} (s={s}, L={L}), {form}")
    else:
        desc = (f"single vector L2C + C2L, N={N}, maxs={maxs} (s={s}, L={L}), "
                f"c_n = s_n/(n+1), {form}")
    return {"workload": desc, "N": N, "maxs": maxs, "s": s, "L": L, "vectors": count,
            "precision": "fp64", "lagrange": lagrange, "l2_flush": "256 MiB write between steps",
            "transforms_per_step": 2 * count}


class Workload:
    """A step: a list of transforms (direction, input, output) on one plan."""

    def __init__(self, name, N, maxs, seed, lagrange=0):
        self.name, self.N, self.maxs, self.lagrange = name, N, maxs, lagrange
        if name == "single":
            self.count = 1
            self.u = sign_decay_input(N, seed)[None, :]
            # L2C and C2L of the same vector
            self.calls = [(0, "u", "o0"), (1, "u", "o1")]
        elif name == "batch":
            self.count = 4096
            self.u = gauss2_lines(self.count, N, seed)
            # L2C of every line, then C2L of the result
            self.calls = [(0, "u", "o0"), (1, "o0", "o1")]
        elif name in ("mixed_batch", "mixed_batch_ref"):
            self.count = 256
            self.u = np.random.default_rng(seed).standard_normal((self.count, N))
            self.calls = [(0, "u", "o0"), (1, "u", "o1")]
        elif name == "mixed_single":
            self.count = 1
            self.u = np.random.default_rng(seed).standard_normal((1, N))
            self.calls = [(0, "u", "o0"), (1, "u", "o1")]
        elif name == "ragged":
            self.Ns = ragged_lengths(2000, seed)
            self.count = len(self.Ns)
            self.total = int(self.Ns.sum())
            rng = np.random.default_rng(seed + 1)
            self.u = rng.uniform(-1.0, 1.0, self.total)[None, :]
            self.calls = [(0, "u", "o0"), (1, "u", "o1")]
            self.coefs_per_step = 2 * self.total
            return
        else:
            raise ValueError(name)
        self.coefs_per_step = 2 * self.count * N

    def config(self):
        return workload_config(self.N, self.maxs, self.name, self.count,
                               getattr(self, "total", None), self.lagrange)

    def cpu_oracle(self, oracle):
        if self.name == "mixed_batch_ref":
            return oracle.Oracle(self.N, self.maxs, 2)
        if self.name == "ragged":
            return oracle.RaggedOracle(self.Ns, self.maxs, 2)
        return oracle.Oracle(self.N, self.maxs, 2, self.lagrange)

    def cpu_call(self, o, src, dst, d):
        if self.name == "ragged":
            o.execute(src[0], dst[0], d)
        elif self.count == 1:
            o.execute(src[0], dst[0], d)
        elif self.name == "mixed_batch_ref":
            o.execute_batch(src, dst, d, self.count, self.N)
        else:
            o.execute_batch(src, dst, d, self.count, self.N)


REF_DIR = os.path.join(REPO, "oracle", "_ref")
REF_LIB = os.path.join(REF_DIR, "libleg2cheb_ref.so")
REF_BATCH = os.path.join(REF_DIR, "libref_batch.so")


class PortCPU:
    """The oracle port of the reference algorithm (oracle/l2c_oracle.c, OpenMP)."""

    kind = "port"

    def __init__(self, wl, threads, why):
        sys.path.insert(0, REPO)
        from oracle import oracle

        oracle.set_threads(threads)
        self.wl, self.o = wl, wl.cpu_oracle(oracle)
        self.note = f"oracle port of the reference algorithm with OpenMP ({why})"

    def call(self, src, dst, d):
        self.wl.cpu_call(self.o, src, dst, d)


class ReferenceCPU:
    """The reference's own execute() (src/C/leg2cheb.c:1299-1500), compiled
    from its unmodified sources into oracle/_ref by oracle/Makefile, called
    through ctypes.  A single vector runs on one plan with every host thread
    (the reference's OpenMP loops and OpenBLAS threads); a batch loops execute
    over the vectors with one plan per OpenMP thread (oracle/ref_batch.c)."""

    kind = "reference"

    def __init__(self, wl, threads):
        import ctypes

        sz, vp = ctypes.c_size_t, ctypes.c_void_p
        self.lib = ctypes.CDLL(REF_LIB, mode=ctypes.RTLD_GLOBAL)
        self.batch = ctypes.CDLL(REF_BATCH)
        self.lib.create_fmm.restype = vp
        self.lib.create_fmm.argtypes = [sz] * 7
        self.lib.execute.restype = sz
        self.lib.execute.argtypes = [vp, vp, vp, sz, sz]
        self.lib.free_fmm.argtypes = [vp]
        self.batch.ref_batch_create.restype = vp
        self.batch.ref_batch_create.argtypes = [sz, vp, sz, sz]
        self.batch.ref_batch_execute.restype = sz
        self.batch.ref_batch_execute.argtypes = [vp, vp, vp, sz]
        self.batch.ref_batch_free.argtypes = [vp]
        self.batch.ref_set_threads.argtypes = [ctypes.c_int, ctypes.c_int]
        self.wl, self.plan, self.handle = wl, None, None
        if wl.count == 1:
            self.plan = self.lib.create_fmm(wl.N, wl.maxs, 18, 2, wl.lagrange, 0, 0)
            if not self.plan:
                raise RuntimeError("reference create_fmm failed")
            omp_t, blas_t = self._pick_threads(threads)
            self.note = (f"the reference's execute() built from its unmodified sources, one plan, "
                         f"{omp_t} OpenMP threads and {blas_t} OpenBLAS threads (the fastest of "
                         f"the settings tried: {self.tried})")
        else:
            Ns = np.full(wl.count, wl.N, dtype=np.uint64)
            self.handle = self.batch.ref_batch_create(wl.count, Ns.ctypes.data, wl.maxs, threads)
            if not self.handle:
                raise RuntimeError("reference batch plans failed")
            self.note = (f"the reference's execute() built from its unmodified sources, looped "
                         f"over the {wl.count} vectors with one plan per OpenMP thread "
                         f"({threads} threads)")

    def _pick_threads(self, threads):
        """The reference's fastest thread setting for this vector: OpenMP on
        every core with OpenBLAS serial or on every core, or OpenMP on half the
        cores (each timed on two steps after one)."""
        u = np.ascontiguousarray(self.wl.u[0])
        out = np.zeros_like(u)
        best, self.tried = None, {}
        for omp_t, blas_t in ((threads, 1), (threads, threads), (max(1, threads // 2), 1)):
            self.batch.ref_set_threads(omp_t, blas_t)
            ts = []
            for _ in range(3):
                out[:] = 0
                t0 = time.perf_counter()
                for d, _, _ in self.wl.calls:
                    self.lib.execute(u.ctypes.data, out.ctypes.data, self.plan, d, 1)
                ts.append(time.perf_counter() - t0)
            t = min(ts[1:])
            self.tried[f"{omp_t}x{blas_t}"] = round(t * 1e3, 2)
            if best is None or t < best[0]:
                best = (t, omp_t, blas_t)
        self.batch.ref_set_threads(best[1], best[2])
        return best[1], best[2]

    def call(self, src, dst, d):
        src = np.ascontiguousarray(src)
        if self.plan:
            self.lib.execute(src.ctypes.data, dst.ctypes.data, self.plan, d, 1)
        else:
            self.batch.ref_batch_execute(self.handle, src.ctypes.data, dst.ctypes.data, d)

    def close(self):
        if self.plan:
            self.lib.free_fmm(self.plan)
            self.plan = None
        if self.handle:
            self.batch.ref_batch_free(self.handle)
            self.handle = None


def cpu_impl(wl, threads):
    """The CPU implementation the reference arm and the CPU baseline time: the
    reference itself where it was built (oracle/_ref) and can run the workload,
    else the oracle port."""
    if wl.name == "ragged":
        # the reference's L2C of an odd N with L >= 1 runs past its arrays
        # (leg2cheb.c:283-294: an unsigned test that never ends the last block's
        # loop), and the list holds odd lengths
        return PortCPU(wl, threads, "the reference itself cannot run odd-length L2C")
    if not (os.path.exists(REF_LIB) and os.path.exists(REF_BATCH)):
        return PortCPU(wl, threads, "the reference was not built on this machine")
    try:
        return ReferenceCPU(wl, threads)
    except (OSError, RuntimeError) as exc:
        return PortCPU(wl, threads, f"the reference build did not load: {exc}")


def cpu_run(wl, seconds, threads):
    """CPU implementation (cpu_impl) on all host cores: the workload's step
    repeated for about `seconds`; returns (coefficients per second, outputs,
    reps, implementation)."""
    impl = cpu_impl(wl, threads)
    bufs = {"u": np.ascontiguousarray(wl.u), "o0": np.zeros_like(wl.u), "o1": np.zeros_like(wl.u)}
    times = []
    t_start = time.perf_counter()
    while True:
        bufs["o0"][:] = 0
        bufs["o1"][:] = 0
        t0 = time.perf_counter()
        for d, src, dst in wl.calls:
            impl.call(bufs[src], bufs[dst], d)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start > seconds and len(times) >= 2:
            break
    return wl.coefs_per_step / statistics.median(times), bufs, len(times), impl


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    wl = Workload(args.workload, args.N, args.maxs, 1, args.lagrange)
    threads = os.cpu_count() or 1
    impl = cpu_impl(wl, threads)
    bufs = {"u": np.ascontiguousarray(wl.u), "o0": np.zeros_like(wl.u), "o1": np.zeros_like(wl.u)}

    def step():
        bufs["o0"][:] = 0
        bufs["o1"][:] = 0
        t0 = time.perf_counter()
        for d, src, dst in wl.calls:
            impl.call(bufs[src], bufs[dst], d)
        return time.perf_counter() - t0

    for _ in range(args.warmup):
        step()
    times = [step() for _ in range(args.steps)]
    t = sum(times) / len(times)
    value = wl.coefs_per_step / t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "coef/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": wl.config(),
        "cpu_baseline": {"value": value, "unit": "coef/s", "cores": threads, "kind": impl.kind,
                         "sample": f"full workload per step ({wl.coefs_per_step} coefficients), "
                                   f"{args.steps} steps; {impl.note}"},
        "e2e": {"value": value, "unit": "coef/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def autotune_plan(plan, calls, count, N):
    """Tune the plan's launch choices for the call shapes the bench times
    (l2c_gpu_autotune; results are the same bits under every choice).  Returns
    the record for the JSON line: per direction the choices, tuned and default
    ms per call, and the tuning time (plan-time work, outside the timed region)."""
    t0 = time.perf_counter()
    shapes = {}
    for d in sorted({c[0] for c in calls}):
        plan.autotune(d, count, N, 1)
        src, text, mt, md = plan.tuned_config(d, count, N, 1)
        shapes[("L2C", "C2L")[d]] = {"choices": text, "ms_per_call": round(mt, 4),
                                     "ms_per_call_default": round(md, 4)}
    return {"seconds": round(time.perf_counter() - t0, 3), "shapes": shapes}


def load_library():
    """Build (if stale) and import the in-tree library front end."""
    sys.path.insert(0, PKG)
    import importlib.util

    spec = importlib.util.spec_from_file_location("l2c_pkg_build", os.path.join(PKG, "build.py"))
    bmod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bmod)
    bmod.build()
    import l2c_gb300

    return l2c_gb300


MIXED_FORM = ("f64 (mixed: far-field, leaf and transfer products on FP16 tensor cores from "
              "exact 9-bit digit slices with exact integer recombination; Lambda and output "
              "accumulation in FP64; near-field band in FP64 (plan 'mixed') or, for the full "
              "blocks of a batch, on the same exact tensor-core scheme (plan 'mixed_tc_band'))")


def compare_mixed(l2c, workload, N, maxs_mixed, steps, warmup, autotune, dev, torch,
                  only=None, maxs_tc=32):
    """Mixed form against plain FP64 on the same inputs (single vector N = 2^22
    or 256 vectors of N = 16384, iid N(0,1), seed 1; L2C and C2L of the same
    input per step).  Plain plans at maxs 16, 32 and 64 (and the mixed plans'
    leaf bounds) are each autotuned and timed; every output is compared with
    the oracle port.  Two mixed plans: 'mixed' (maxs_mixed) keeps the near-field
    band in FP64 (L2C_MZ_BAND=0), 'mixed_tc_band' (maxs_tc) runs a batch's full
    band blocks on the tensor cores too.  Returns the record: per plan ms,
    coef/s, launches and phases; errors per direction; the speed-ups of the
    fastest mixed plan and of the FP64-band one against the fastest plain plan."""
    import ctypes

    wl = Workload(workload, N, maxs_mixed, 1)
    N, count = wl.N, wl.count
    du = torch.from_numpy(np.ascontiguousarray(wl.u)).to(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def time_plan(plan):
        stream = torch.cuda.ExternalStream(plan.stream, device=dev)
        outs = [torch.zeros_like(du), torch.zeros_like(du)]

        def step():
            with torch.cuda.stream(stream):
                flush.fill_(1)
                outs[0].zero_()
                outs[1].zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            plan.execute_async(du, outs[0], 0, count, N, 1)
            plan.execute_async(du, outs[1], 1, count, N, 1)
            e1.record(stream)
            return e0, e1

        for _ in range(warmup):
            step()
        plan.synchronize()
        l0 = l2c.cuda_abi().l2c_gpu_launch_count(plan._gpu)
        evs = [step() for _ in range(steps)]
        plan.synchronize()
        launches = l2c.cuda_abi().l2c_gpu_launch_count(plan._gpu) - l0
        ms = sum(a.elapsed_time(b) for a, b in evs) / len(evs)
        # per-phase CUDA events in a separate pass (graph replay off while profiling)
        abi = l2c.cuda_abi()
        abi.l2c_gpu_profile(plan._gpu, 1)
        nprof = max(1, min(steps, 20))
        for _ in range(nprof):
            step()
        plan.synchronize()
        pms = (ctypes.c_double * 8)()
        pl = (ctypes.c_size_t * 8)()
        abi.l2c_gpu_profile_read(plan._gpu, pms, pl)
        abi.l2c_gpu_profile(plan._gpu, 0)
        names = ["gather", "near", "leaf_up", "tree_up", "far", "tree_down", "leaf_down", "direct"]
        phases = {names[i]: round(pms[i] / nprof, 4) for i in range(8) if pl[i]}
        return ms, [o.cpu().numpy() for o in outs], launches, phases

    def time_e2e(plan):
        """The same step through execute_batched() with pinned host buffers
        (input and zeroed outputs read over the host link, results written
        back, per call)."""
        hu = torch.from_numpy(np.ascontiguousarray(wl.u)).pin_memory()
        ho = [torch.zeros_like(hu).pin_memory(), torch.zeros_like(hu).pin_memory()]
        ts = []
        for it in range(warmup + min(steps, 20)):
            ho[0].zero_()
            ho[1].zero_()
            t0 = time.perf_counter()
            plan.execute_batched(hu, ho[0], 0, count, N, 1)
            plan.execute_batched(hu, ho[1], 1, count, N, 1)
            if it >= warmup:
                ts.append(time.perf_counter() - t0)
        st = sum(ts) / len(ts)
        nbytes = 8 * wl.u.size
        return {"value": 2 * count * N / st, "unit": "coef/s", "h2d_bytes_per_step": 4 * nbytes,
                "d2h_bytes_per_step": 2 * nbytes, "ms_per_step": st * 1e3}

    results = {}
    plain_bounds = sorted({16, 32, 64, maxs_mixed, maxs_tc})
    for name, maxs, mixed, band in ([(f"plain_maxs{m}", m, False, None) for m in plain_bounds]
                                    + [("mixed", maxs_mixed, True, "0"),
                                       ("mixed_tc_band", maxs_tc, True, "1")]):
        if only and name not in only:
            continue
        t_plan0 = time.perf_counter()
        saved = os.environ.get("L2C_MZ_BAND")
        if band is not None:
            os.environ["L2C_MZ_BAND"] = band  # read when the plan is created
        try:
            plan = l2c.Plan(N, maxs, mixed=mixed)
        finally:
            if saved is None:
                os.environ.pop("L2C_MZ_BAND", None)
            else:
                os.environ["L2C_MZ_BAND"] = saved
        plan_ms = (time.perf_counter() - t_plan0) * 1e3
        tuned = autotune_plan(plan, ((0,), (1,)), count, N) if autotune else None
        ms, outs, launches, phases = time_plan(plan)
        results[name] = {"maxs": maxs, "s": plan.s, "L": plan.L, "ms_per_step": ms,
                         "value": 2 * count * N / (ms * 1e-3), "launches": launches,
                         "phases_ms_per_step": phases, "autotune": tuned,
                         "create_fmm_ms": round(plan_ms, 3),
                         "flops": plan.flops(0) + plan.flops(1), "outs": outs}
        if mixed:
            results[name]["e2e"] = time_e2e(plan)
        plan.close()
    # accuracy against the oracle port (FP64) on the same inputs, every vector
    sys.path.insert(0, REPO)
    from oracle import oracle

    oracle.set_threads(os.cpu_count() or 1)
    errs = {}
    for name, r in results.items():
        o = oracle.Oracle(N, r["maxs"], 2)
        e = []
        for d in (0, 1):
            want = np.zeros_like(wl.u)
            if count == 1:
                o.execute(np.ascontiguousarray(wl.u[0]), want[0], d)
            else:
                o.execute_batch(np.ascontiguousarray(wl.u), want, d, count, N)
            den = np.max(np.abs(want), axis=1)
            e.append(float(np.max(np.max(np.abs(r["outs"][d] - want), axis=1) / den)))
        o.close()
        errs[name] = {"l2c": e[0], "c2l": e[1]}
        del r["outs"]
    mixed_names = [k for k in results if k.startswith("mixed")]
    if not mixed_names or not any(k.startswith("plain") for k in results):
        return {"plans": results, "max_rel_err_vs_oracle": errs,
                "e2e_mixed": {k: results[k]["e2e"] for k in mixed_names}}
    best_mixed = min((results[k]["ms_per_step"], k) for k in mixed_names)[1]
    mixed = results[best_mixed]
    e2e_mixed = mixed["e2e"]
    best_plain = min((results[k]["ms_per_step"], k) for k in results if k.startswith("plain"))
    return {
        "workload": (f"mixed vs plain FP64, {'single vector' if count == 1 else str(count) + ' vectors'} "
                     f"of N={N}, iid N(0,1), L2C and C2L of the same input per step"),
        "N": N, "vectors": count, "maxs_mixed": maxs_mixed, "steps": steps, "warmup": warmup,
        "best_mixed": best_mixed,
        "ms_per_step_mixed": mixed["ms_per_step"], "value_mixed": mixed["value"],
        "ms_per_step_best_plain": best_plain[0], "best_plain": best_plain[1],
        "speedup_vs_best_plain": best_plain[0] / mixed["ms_per_step"],
        # the mixed form as the benchmark's configuration describes it (band in FP64)
        "speedup_vs_best_plain_fp64_band": (best_plain[0] / results["mixed"]["ms_per_step"]
                                            if "mixed" in results else None),
        "speedup_vs_plain_maxs64": results["plain_maxs64"]["ms_per_step"] / mixed["ms_per_step"],
        "max_rel_err_vs_oracle": errs,
        "error_note": "relative max-norm per vector (max over the batch), per direction, "
                      "against the oracle port (FP64) on the same inputs",
        "plans": results, "e2e_mixed": e2e_mixed,
        "l2_flush": "256 MiB write between steps", "dtype": MIXED_FORM,
    }


def run_mixed(args):
    """--workload mixed_single | mixed_batch: a line whose value is the mixed
    form's throughput, with the plain plans beside it (compare_mixed)."""
    import torch

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    l2c = load_library()
    peak = measured_fp64_peak(torch, dev)
    clocks = ClockSampler(0)
    clocks.start()
    only = set(args.mixed_plans.split(",")) if args.mixed_plans else None
    rec = compare_mixed(l2c, args.workload, args.N, args.maxs_mixed, args.steps, args.warmup,
                        args.autotune, dev, torch, only, args.maxs_mixed_tc)
    clk = clocks.stop()
    if "speedup_vs_best_plain" not in rec:  # a subset of the plans (profiling runs)
        print(json.dumps({"plans": rec["plans"], "errors": rec["max_rel_err_vs_oracle"],
                          "e2e_mixed": rec["e2e_mixed"], "clocks": clk}))
        return 0
    mixed = rec["plans"][rec["best_mixed"]]
    line = {
        "metric": METRIC, "value": mixed["value"], "unit": "coef/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": mixed["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": MIXED_FORM, "data": "synthetic (seeded iid N(0,1))",
        "config": {"workload": rec["workload"], "N": rec["N"], "vectors": rec["vectors"],
                   "maxs_mixed": args.maxs_mixed, "maxs_mixed_tc": args.maxs_mixed_tc,
                   "best_mixed": rec["best_mixed"], "l2_flush": "256 MiB write between steps"},
        "plans": rec["plans"],
        "max_rel_err_vs_oracle": rec["max_rel_err_vs_oracle"],
        "speedup_mixed_vs_plain_maxs64": rec["speedup_vs_plain_maxs64"],
        "speedup_mixed_vs_best_plain": rec["speedup_vs_best_plain"],
        "speedup_mixed_fp64_band_vs_best_plain": rec["speedup_vs_best_plain_fp64_band"],
        "best_plain": rec["best_plain"],
        "clocks": clk,
        "fp64_peak_tflops_measured": peak,
        "gpu_launches": int(mixed["launches"]),
        "e2e": rec["e2e_mixed"],
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="single",
                    choices=["single", "batch", "ragged", "mixed_single", "mixed_batch"])
    ap.add_argument("--mixed-plans", default=None,
                    help="mixed_* workloads: comma-separated subset of the plans to time "
                         "(plain_maxs16, plain_maxs32, plain_maxs64, mixed, mixed_tc_band), "
                         "for profiling")
    ap.add_argument("--maxs-mixed", type=int, default=16,
                    help="leaf size bound of the mixed-form plan with the FP64 band")
    ap.add_argument("--maxs-mixed-tc", type=int, default=32,
                    help="leaf size bound of the mixed-form plan with the tensor-core band")
    ap.add_argument("--N", type=int, default=None)
    ap.add_argument("--maxs", type=int, default=64)
    ap.add_argument("--precompute", type=int, default=0,
                    help="1: keep the near-field band weights in device memory (create_fmm's "
                         "precompute argument)")
    ap.add_argument("--lagrange", type=int, default=0, choices=[0, 1],
                    help="1: the nodal form (create_fmm's lagrange argument; single, batch)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true",
                    help="leave out the mixed-vs-plain record of the default line")
    ap.add_argument("--autotune", type=int, default=1, choices=[0, 1],
                    help="tune each plan's launch choices for the timed call shapes first "
                         "(same bits under every choice; tuning time reported, not timed)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.N is None:
        args.N = {"single": 1 << 20, "batch": 1024, "ragged": 1024, "mixed_single": 1 << 22,
                  "mixed_batch": 16384}[args.workload]
    if args.lagrange and args.workload not in ("single", "batch"):
        ap.error("--lagrange 1 applies to the single and batch workloads")
    if args.workload.startswith("mixed"):
        if args.impl == "reference":
            args.workload = "single" if args.workload == "mixed_single" else "mixed_batch_ref"
        else:
            return run_mixed(args)
    if args.impl == "reference":
        return run_reference(args)

    import torch

    rank, world, local = rank_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ranks = Ranks(world, "nccl", dev)
    barrier, max_over_ranks = ranks.barrier, ranks.max

    if rank == 0:
        load_library()
    barrier()
    import ctypes

    import l2c_gb300 as l2c

    abi = l2c.cuda_abi()
    wl = Workload(args.workload, args.N, args.maxs, 1 + rank, args.lagrange)
    N, maxs, count = wl.N, wl.maxs, wl.count
    ragged = wl.name == "ragged"
    if ragged:
        plan = l2c.RaggedPlan(wl.Ns, maxs, precompute=args.precompute)
    else:
        plan = l2c.Plan(N, maxs, precompute=args.precompute, lagrange=args.lagrange)
    stream = torch.cuda.ExternalStream(plan.stream, device=dev)
    dbuf = {"u": torch.from_numpy(np.ascontiguousarray(wl.u)).to(dev)}
    dbuf["o0"] = torch.zeros_like(dbuf["u"])
    dbuf["o1"] = torch.zeros_like(dbuf["u"])
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    peak = measured_fp64_peak(torch, dev)
    hbm_peak = hbm_peak_gbs()

    def step(pl=None, st=None):
        pl, st = pl or plan, st or stream
        with torch.cuda.stream(st):
            flush.fill_(1)
            dbuf["o0"].zero_()
            dbuf["o1"].zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for d, src, dst in wl.calls:
            if ragged:
                pl.execute_async(dbuf[src], dbuf[dst], d)
            else:
                pl.execute_async(dbuf[src], dbuf[dst], d, count, N, 1)
        e1.record(st)
        return e0, e1

    def phase_pass(pl, st):
        """args.steps steps with per-phase CUDA events (direct launches)."""
        abi.l2c_gpu_profile(pl._gpu, 1)
        evs = [step(pl, st) for _ in range(args.steps)]
        pl.synchronize()
        ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in evs) / len(evs))
        pms = (ctypes.c_double * 8)()
        pl_n = (ctypes.c_size_t * 8)()
        abi.l2c_gpu_profile_read(pl._gpu, pms, pl_n)
        abi.l2c_gpu_profile(pl._gpu, 0)
        names = ["gather", "near", "leaf_up", "tree_up", "far", "tree_down", "leaf_down", "direct"]
        return ms, {names[i]: {"ms_per_step": pms[i] / args.steps,
                               "launches_per_step": pl_n[i] / args.steps}
                    for i in range(8) if pl_n[i]}

    tuned = None
    if args.autotune and ragged:
        t_tune0 = time.perf_counter()
        shapes = {}
        for d in sorted({c[0] for c in wl.calls}):
            plan.autotune(d)
            src, text, mt, md = plan.tuned_config(d)
            shapes[("L2C", "C2L")[d]] = {"choices": text, "ms_per_call": round(mt, 4),
                                         "ms_per_call_default": round(md, 4)}
        tuned = {"seconds": round(time.perf_counter() - t_tune0, 3), "shapes": shapes}
    elif args.autotune:
        tuned = autotune_plan(plan, wl.calls, count, N)
    for _ in range(args.warmup):
        step()
    plan.synchronize()
    torch.cuda.synchronize()

    # ---- timed region (device resident, each call shape replayed as a CUDA graph) ----
    launches0 = abi.l2c_gpu_launch_count(plan._gpu) if not ragged else plan.launch_count()
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
    launches = (abi.l2c_gpu_launch_count(plan._gpu) if not ragged else plan.launch_count()) - launches0
    ms_step = max_over_ranks(sum(a.elapsed_time(b) for a, b in evs) / len(evs))
    value = aggregate_value(wl.coefs_per_step, world, ms_step)

    # ---- the same K steps again with per-phase CUDA events (direct launches) ----
    phases, phases_iso = {}, {}
    ms_prof = None
    plan_ms = None
    if not ragged:
        ms_prof, phases = phase_pass(plan, stream)
        # the band alone: a plan whose band runs on its own stream, before the
        # far-field chain (in the step above it shares the SMs with the chain)
        os.environ["L2C_OVERLAP"] = "0"
        try:
            t_plan0 = time.perf_counter()
            plan_iso = l2c.Plan(N, maxs, precompute=args.precompute, lagrange=args.lagrange)
            plan_ms = (time.perf_counter() - t_plan0) * 1e3
        finally:
            del os.environ["L2C_OVERLAP"]
        st_iso = torch.cuda.ExternalStream(plan_iso.stream, device=dev)
        for _ in range(2):
            step(plan_iso, st_iso)
        plan_iso.synchronize()
        _, phases_iso = phase_pass(plan_iso, st_iso)
        plan_iso.close()

    # ---- e2e through execute() with pinned host buffers ----
    hbuf = {"u": torch.from_numpy(np.ascontiguousarray(wl.u)).pin_memory()}
    hbuf["o0"] = torch.zeros(wl.u.shape, dtype=torch.float64).pin_memory()
    hbuf["o1"] = torch.zeros(wl.u.shape, dtype=torch.float64).pin_memory()
    e2e_t = []
    for it in range(args.warmup + min(args.steps, 50)):
        hbuf["o0"].zero_()
        hbuf["o1"].zero_()
        t0 = time.perf_counter()
        for d, src, dst in wl.calls:
            if ragged:
                plan(hbuf[src], hbuf[dst], d)
            else:
                plan.execute_batched(hbuf[src], hbuf[dst], d, count, N, 1)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            e2e_t.append(dt)
    e2e_step = max_over_ranks(sum(e2e_t) / len(e2e_t))
    e2e_value = wl.coefs_per_step * world / e2e_step
    nbytes = 8 * wl.u.size

    # ---- roofline of the band kernel (the dominant FP64 kernel) ----
    L, s, _ = l2c.geometry(N, maxs) if not ragged else (None, None, None)
    roof = None
    if ragged:
        total_flops = sum(plan.flops(d) for d, _, _ in wl.calls)
        achieved = total_flops / (ms_step * 1e-3) / 1e12
        roof = {"bound": "fp64", "pipe": "fp64", "kernel": "whole step (all ragged kernels)",
                "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": None, "peak_source": FP64_PEAK_SOURCE}
    if "near" in phases_iso and L >= 1:
        nf = sum(near_flops(N, s, d) for d, _, _ in wl.calls) * count / len(wl.calls)

        def band_rate(ph):
            # the band of one call (its launches: the full blocks, then the last block)
            per_call = ph["near"]["ms_per_step"] / len(wl.calls)
            return per_call, nf / (per_call * 1e-3) / 1e12, ph["near"]["launches_per_step"] / len(wl.calls)

        ms_call, achieved, launches_call = band_rate(phases_iso)
        ms_call_step, achieved_step, _ = band_rate(phases)
        # DRAM bytes of one call's band from the committed ncu summary of this
        # same command (dram__bytes_read.sum + dram__bytes_write.sum of its
        # launches, mean of the L2C and C2L calls); other workloads were not
        # captured.
        captured = (wl.name == "single" and N == 1 << 20 and maxs == 64
                    and args.precompute == 0 and args.lagrange == 0)
        traffic = profile_traffic(BAND_PROFILE, calls=2) if captured else None
        kernel = ("band: " + ("k_band_tile (full blocks) + k_near (last block)" if count >= 64 and s % 8 == 0
                              else "k_near_rows (full blocks) + k_near (last block)" if count == 1 and s % 8 == 0
                              else "k_near / k_near_pair"))
        roof = {"bound": "fp64", "pipe": "fp64", "kernel": kernel,
                "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": traffic,
                "traffic_unit": "DRAM bytes per call (the call's band launches)",
                "traffic_source": BAND_PROFILE if traffic is not None else None,
                "algorithmic_bytes_per_call": 24 * N * count,
                "peak_source": FP64_PEAK_SOURCE,
                "flops_per_call": nf, "ms_per_call": ms_call, "launches_per_call": launches_call,
                "timing": "the band's launches of each call timed with CUDA events on their "
                          "stream, in a pass of the same workload with the band on the plan's "
                          "stream (the band alone on the GPU)",
                "achieved_in_step": achieved_step, "frac_in_step": achieved_step / peak,
                "ms_per_call_in_step": ms_call_step,
                "in_step_note": "in the timed step the band runs on a second stream beside "
                                "the far-field chain, whose kernels have scheduling priority",
                "note": "reference flop count of directM/directL (3 per band term); a term "
                        "costs 2 FP64 issue slots (DMUL+DFMA), or 1 (DFMA) when the band "
                        "reads its weights from a table (precompute=1, and batches whose "
                        "table is no larger than their input); with a table, or with one "
                        "weight shared by 8 vectors, frac can pass 1"}
    if not ragged:
        total_flops = sum(plan.flops(d) for d, _, _ in wl.calls) * count

    line = {
        "metric": METRIC, "value": value, "unit": "coef/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": dict(wl.config(), precompute=args.precompute),
        "e2e": {"value": e2e_value, "unit": "coef/s",
                "h2d_bytes_per_step": len(wl.calls) * 2 * nbytes,
                "d2h_bytes_per_step": len(wl.calls) * nbytes, "ms_per_step": e2e_step * 1e3},
        "gpu_launches": int(launches),
        "clocks": clk,
        "roofline": roof,
        "phases": phases,
        "ms_per_step_phase_profiled": ms_prof,
        "phase_roofline": (phase_roofline(wl, L, s, plan.Nb, phases_iso, peak, hbm_peak[0],
                                          args.lagrange) if not ragged and L >= 1 else None),
        "phase_roofline_note": ("per FMM step, each timed alone (band on the plan's stream); "
                                "flops: the reference's count (band: 3 per term, 2 FP64 "
                                "instructions); bytes: algorithmic DRAM bytes; peaks: FP64 "
                                "DGEMM measured in this run, HBM " + hbm_peak[1]),
        "fp64_ref_tflops_whole_step": total_flops / (ms_step * 1e-3) / 1e12,
        "wall_s_timed_region": t_wall,
        "plan": ({"L": L, "s": s, "Nb": plan.Nb, "create_fmm_ms": plan_ms} if not ragged
                 else {"vectors": count}),
        "autotune": tuned,
    }
    got = {k: dbuf[k].cpu().numpy() for k in ("o0", "o1")}
    if wl.name == "batch":
        line["roundtrip_rel_err"] = float(np.max(np.abs(got["o1"] - wl.u)) / np.max(np.abs(wl.u)))

    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        cpu_value, outs, reps, impl = cpu_run(wl, args.cpu_seconds, threads)
        line["cpu_baseline"] = {
            "value": cpu_value, "unit": "coef/s", "cores": threads, "kind": impl.kind,
            "sample": f"{reps} repetitions of the full step ({wl.coefs_per_step} coefficients), "
                      f"median; {impl.note}"}
        line["max_rel_err_vs_oracle"] = {
            name: float(np.max(np.abs(got[k] - outs[k])) / np.max(np.abs(outs[k])))
            for name, k in (("l2c", "o0"), ("c2l", "o1"))}
        line["max_rel_err_vs"] = impl.note
    if (rank == 0 and world == 1 and not ragged and not args.no_mixed
            and wl.name == "single" and args.lagrange == 0):
        # the metric's second half: mixed form against the fastest plain plan,
        # on the two mixed-precision workloads, each with its own clock record
        line["mixed"] = {}
        for key, wname, n_mixed in (("batch", "mixed_batch", 16384),
                                    ("single", "mixed_single", 1 << 22)):
            clk_m = ClockSampler(local)
            clk_m.start()
            rec = compare_mixed(l2c, wname, n_mixed, args.maxs_mixed, min(args.steps, 20),
                                args.warmup, args.autotune, dev, torch, None, args.maxs_mixed_tc)
            rec["clocks"] = clk_m.stop()
            line["mixed"][key] = rec
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
