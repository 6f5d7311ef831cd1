"""Benchmark: DiffusionLenia steps per second on a GB300.

Workload: one 2048x2048 creature, 3 channels, 9 kernels over every
(input, output) pair, seeded synthetic ring kernels (the reference ships no
creatures), the whole step captured in one CUDA graph.  A benchmark step is
one DiffusionLenia step; the metric is cell-updates/s = n^2 * steps / time,
summed over ranks.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``--impl reference`` times the CPU implementation of the same step (the
FP32 C restatement of ml-rs/example.rs, all host threads) on a bounded
sample, since the reference's own GPU path needs wgpu/Vulkan, which is
unavailable on this machine, and its Rust CPU program cannot be built here.
Under torchrun, ranks run independent replicas (no data exchange); rank 0
prints one JSON line.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_GRID, C_CH, K_KER = 2048, 3, 9
METRIC = "cell-updates/s (DiffusionLenia fwd step, 2048^2, C=3, K=9)"
UNIT = "cell-updates/s"
WORKLOAD = "DiffusionLenia 2048x2048, 3 channels, 9 kernels (all pairs), 1 creature, " \
           "8 steps per CUDA graph (per-channel launches on forked streams)"


def bytes_per_px(C, K):
    """Algorithmic bytes per grid point per step (fp32 state, complex64 half
    spectra, each source spectrum read once) for the pass structure the
    performance target is defined on: row R2C read+write 8C, a forward column
    pass read+write 8C, the inverse column pass reading each source spectrum
    once 4C and each kernel spectrum with its intermediate write 8K, the C2R
    row read 4K, the affinity write 4C and the fused diffusion 12C."""
    return 36 * C + 12 * K


def bytes_per_px_as_built(C, K, real=False):
    """The same for the passes this library runs: the forward column FFT is
    fused into the column convolution, so its 8C never reach HBM (row pass 8C,
    column pass 4C + 8K, inverse row pass 4K + 4C, diffusion 12C).  With real
    kernel spectra (point-symmetric kernels) the column pass reads 2 instead
    of 4 bytes per grid point and kernel: 28C + 10K."""
    return 28 * C + (10 if real else 12) * K


def col_conv_bytes_per_px(C, K, real=False):
    """k_col_conv: read the row spectra once (4C), read each kernel's half
    spectrum (4K complex, 2K real) and write its column-inverted product
    (4K)."""
    return 4 * C + (6 if real else 8) * K


# Algorithmic bytes per grid point of each step kernel, in the order of
# profile_kernels' split (row_r2c, col_conv, row_c2r_growth, diffusion).
KERNEL_NAMES = ("k_row_r2c", "k_col_conv", "k_row_c2r_growth", "k_diffusion")


def kernel_bytes_per_px(C, K, real=False):
    return (8 * C,                       # read the state, write the row spectra
            col_conv_bytes_per_px(C, K, real),
            4 * K + 4 * C,               # read each U, write A
            12 * C)                      # read A and the state, write the new state


def roofline_object(kms, n, C, K, peak, peak_kind, traffic=None, real=False):
    """The `roofline` object of the bench line: every step kernel's
    algorithmic bytes per launch (kernel_bytes_per_px x n^2) over its
    measured duration (kms, ms per step, in KERNEL_NAMES order) against the
    peak, and the kernel with the largest device time reported on top.
    `traffic` maps "<kernel>_<n>" to an ncu capture's DRAM bytes per launch;
    `real`: the column pass reads real kernel spectra."""
    traffic = traffic or {}
    px = n * n
    per_kernel = []
    for name, b, t in zip(KERNEL_NAMES, kernel_bytes_per_px(C, K, real), kms):
        ach = b * px / (t / 1e3) / 1e9
        per_kernel.append({"kernel": name, "algorithmic_bytes": b * px, "kernel_ms": t,
                           "achieved": ach, "frac": ach / peak,
                           "traffic": traffic.get(f"{name}_{n}", {}).get("dram_bytes_per_launch")})
    top = max(per_kernel, key=lambda r: r["kernel_ms"])
    return {"bound": "hbm", "kernel": top["kernel"], "achieved": top["achieved"], "peak": peak,
            "unit": "GB/s", "frac": top["frac"], "traffic": top["traffic"],
            "algorithmic_bytes": top["algorithmic_bytes"], "kernel_ms": top["kernel_ms"],
            "peak_source": peak_kind, "selection": "the step kernel with the largest device time",
            "kernels": per_kernel}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms.  Each
    sample carries nvidia-smi's own timestamp: its output reaches the pipe in
    bursts, so the arrival time would misplace short windows."""
    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        import datetime
        # nvidia-smi prints local wall-clock time; map it to perf_counter
        offset = time.time() - time.perf_counter()
        for line in self.proc.stdout:
            f = [x.strip() for x in line.split(",")]
            t = time.perf_counter()
            try:
                t = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp() - offset
            except (ValueError, IndexError):
                pass
            self.rows.append((t, f[1:]))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self, t0=None, t1=None, busy=None):
        """Median SM clock, its maximum and the throttle reasons seen in
        [t0, t1].  A timed region shorter than the 100 ms sampling period
        holds no sample; then the samples over `busy` = (start, end, label),
        a span in which the GPU ran this program's work, stand in, and
        `window` says so."""
        def pick(a, b):
            return [r for t, r in self.rows if (a is None or t >= a) and (b is None or t <= b)]
        rows, window = pick(t0, t1), "timed region"
        if not rows and busy is not None:
            rows, window = pick(busy[0], busy[1]), f"GPU-busy span: {busy[2]}"
        if not rows:
            why = ("nvidia-smi printed no sample (the run may be shorter than its start-up)"
                   if self.proc else "nvidia-smi unavailable")
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0,
                    "window": window, "note": why}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if len(r) > 5 + i and r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows), "window": window}


def rank_info():
    """(world, rank, local rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def dist_setup(n_gpus, backend=None):
    """One process per GPU (replicas): NCCL on GPUs, gloo otherwise.  Only the
    timing max-reduce and barriers cross ranks."""
    world, rank, local = rank_info()
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = backend or ("nccl" if torch.cuda.is_available() else "gloo")
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local, dist


def max_over_ranks(x, dist, world):
    if dist is None or world == 1:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist, world):
    if dist is not None and world > 1:
        dist.barrier()


def cpu_baseline(cr, budget_s=20.0, nthreads=None, forms=True):
    """The FP32 C restatement of example.rs (faithful: FFT per kernel), all
    host threads, one step of the full workload (a bounded sample).  With
    forms, one step more in each of the other forms: one thread (example.rs
    is serial) and FP64, each timed once, and the torch CPU model
    (train/diff_lenia_org.py's step, restated in oracle/autograd_ref.py) in
    FP32 on torch's own threads."""
    from oracle import oracle as O
    nthreads = nthreads or os.cpu_count() or 1
    st = cr.seed.astype(np.float32)
    ks = cr.kspec.astype(np.complex128)
    args = (cr.c0, cr.c1, cr.mu.astype(np.float64), cr.sigma.astype(np.float64),
            cr.weights.astype(np.float64), cr.temp)
    times = []
    t_start = time.perf_counter()
    while True:
        t0 = time.perf_counter()
        st, _, _ = O.step_c(st, ks, *args, dtype=np.float32, faithful=True, nthreads=nthreads)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start > budget_s or len(times) >= 3:
            break
    t = min(times)
    out = {"value": cr.n * cr.n / t, "unit": UNIT, "cores": nthreads, "kind": "port",
           "sample": f"{len(times)} step(s) of the {cr.n}^2 C={cr.C} K={cr.K} workload, "
                     f"f32 C port of example.rs (FFT per kernel), OpenMP, best {t:.2f} s/step"}
    if forms:
        rows = [{"threads": nthreads, "dtype": "f32", "s_per_step": round(t, 3)}]
        for r in rows:
            r["impl"] = "C port of example.rs"
        for dt, nt in ((np.float64, nthreads), (np.float32, 1), (np.float64, 1)):
            t0 = time.perf_counter()
            O.step_c(cr.seed.astype(dt), ks, *args, dtype=dt, faithful=True, nthreads=nt)
            rows.append({"threads": nt, "dtype": "f32" if dt == np.float32 else "f64",
                         "impl": "C port of example.rs",
                         "s_per_step": round(time.perf_counter() - t0, 3)})
        try:
            import torch
            from oracle import autograd_ref as R
        except ImportError:
            torch = None
        if torch is not None:
            xt = torch.tensor(np.asarray(cr.seed, np.float32))
            kt = torch.tensor(np.asarray(cr.kspec, np.complex64))
            with torch.no_grad():
                t0 = time.perf_counter()
                R.step(xt, kt, cr.c0, cr.c1, cr.mu, cr.sigma, cr.weights, cr.temp)
                rows.append({"threads": torch.get_num_threads(), "dtype": "f32",
                             "impl": "torch CPU (train/diff_lenia_org.py step)",
                             "s_per_step": round(time.perf_counter() - t0, 3)})
        for r in rows:
            r["cell_updates_per_s"] = cr.n * cr.n / r["s_per_step"]
        out["forms"] = rows
    return out


def oracle_step_error(x, y, cr, nthreads=None):
    """Max-abs difference between a GPU step (x -> y) and the FP64 oracle's
    step from the same state x (the C restatement of example.rs, all host
    threads)."""
    from oracle import oracle as O
    ref, _, _ = O.step_c(np.asarray(x, np.float64), cr.kspec.astype(np.complex128), cr.c0,
                         cr.c1, cr.mu.astype(np.float64), cr.sigma.astype(np.float64),
                         cr.weights.astype(np.float64), cr.temp,
                         nthreads=nthreads or os.cpu_count() or 1)
    return float(np.abs(np.asarray(y, np.float64) - ref).max())


def sample_step(sim):
    """(state, state after one more step) of a world, on the host."""
    x = sim.state()
    sim.iterate()
    return x, sim.state()


def step_errors(pairs, cr):
    """Per-step max-abs errors of the sampled GPU steps against the FP64
    oracle (teacher-forced: each oracle step starts from the GPU's state)."""
    out = {}
    for label, (x, y) in pairs.items():
        out[label] = oracle_step_error(x, y, cr)
    return {"max_abs": max(out.values()), "bar": 1e-5, "steps": out,
            "how": "teacher-forced: a GPU step against the FP64 oracle's step from the same "
                   "state, at the points of the run named in `steps`"}


def run_reference(args):
    # rank 0 alone times the CPU reference; the other ranks exit without work
    # (and without joining a process group)
    world, rank, _ = rank_info()
    if rank != 0:
        return 0
    from cella_nova_gb300.creature import make_creature
    from oracle import oracle as O
    O.build()
    cr = make_creature(N_GRID, C_CH, seed=2048, temp=1.0)
    nthreads = os.cpu_count() or 1
    st = cr.seed.astype(np.float32)
    ks = cr.kspec.astype(np.complex128)
    a = (cr.c0, cr.c1, cr.mu.astype(np.float64), cr.sigma.astype(np.float64),
         cr.weights.astype(np.float64), cr.temp)
    # the same warm-up count as the GPU arm, within a bounded time
    warm, tw = 0, time.perf_counter()
    while warm < args.warmup and time.perf_counter() - tw < 60.0:
        st, _, _ = O.step_c(st, ks, *a, dtype=np.float32, faithful=True, nthreads=nthreads)
        warm += 1
    budget = 150.0
    done, t0 = 0, time.perf_counter()
    while done < args.steps:
        st, _, _ = O.step_c(st, ks, *a, dtype=np.float32, faithful=True, nthreads=nthreads)
        done += 1
        if time.perf_counter() - t0 > budget:
            break
    el = time.perf_counter() - t0
    value = N_GRID * N_GRID * done / el
    sample = (f"{done} of {args.steps} requested steps (150 s budget) after {warm} warm-up "
              f"steps, f32 C port of example.rs, OpenMP {nthreads} threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": done, "warmup": warm,
        "ms_per_step": 1e3 * el / done, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(world), "device": "host CPU",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(world):
    """The `config` object of both arms' lines (the same workload)."""
    return {"workload": WORKLOAD, "n": N_GRID, "channels": C_CH, "kernels": K_KER,
            "parallelism": f"replicas x{world}",
            "l2": "no flush: each step streams ~0.75 GB (> 129 MB L2)"}


def load_traffic():
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def run_ours(args):
    import torch
    world, rank, local, dist = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    from cella_nova_gb300 import GpuMaceLenia
    from cella_nova_gb300.creature import make_creature

    sampler = ClockSampler(local)
    sampler.start()
    t_busy0 = time.perf_counter()
    cr = make_creature(N_GRID, C_CH, seed=2048 + rank, temp=1.0)
    sim = GpuMaceLenia.from_creature(cr)
    real = sim.kernels_real()
    px = N_GRID * N_GRID
    checks = {}
    mass0 = sim.mass_f64()
    checks["step 1 (from the seed)"] = sample_step(sim)
    tuned = None
    if args.variants:
        sim.set_variants([int(v) for v in args.variants.split(",")])
        tuned = {"variants": sim.variants(), "ms": None, "how": "--variants"}
    elif not args.no_autotune:
        chosen, tms = sim.autotune(reps=10)
        tuned = {"variants": chosen, "ms": np.round(tms, 4).tolist(),
                 "graph_layout": sim.graph_layout()}
    stream = torch.cuda.ExternalStream(sim.stream())

    # warm-up, then K timed graph launches between barriers + syncs
    warm = max(args.warmup, 3)
    sim.run_steps(warm)
    sim.synchronize()
    checks["after the warm-up"] = sample_step(sim)
    barrier(dist, world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    t_wall0 = time.perf_counter()
    e0.record(stream)
    sim.run_steps(args.steps)
    e1.record(stream)
    e1.synchronize()
    t_wall1 = time.perf_counter()
    torch.cuda.synchronize()
    barrier(dist, world)
    ms_local = e0.elapsed_time(e1)
    ms = max_over_ranks(ms_local, dist, world)
    checks["after the timed steps"] = sample_step(sim)

    # per-kernel device time with events between kernels (same stream)
    prof_steps = min(max(args.steps, 8), 256)
    kms = sim.profile_kernels(prof_steps)
    sim.synchronize()
    checks[f"after the kernel profile ({prof_steps} more steps)"] = sample_step(sim)
    mass1 = sim.mass_f64()
    total_steps = 1 + warm + 1 + args.steps + 1 + prof_steps + 1
    drift = {"steps": total_steps, "max_rel": float(np.abs(mass1 / mass0 - 1).max()),
             "reduction": "FP64 on the GPU"}
    t_busy1 = time.perf_counter()

    # end to end through the public API with host buffers: per step, upload
    # the state (f64, as upload_channel takes it) from pinned memory, step,
    # download the f32 state
    e2e = None
    if not args.no_e2e:
        e2e = e2e_run(sim, cr, args, dist, world)
    clocks = sampler.summary(t_wall0, t_wall1,
                             (t_busy0, t_busy1, "autotune, warm-up, timed and profiled steps"))

    cpu = step_err = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(cr)
        step_err = step_errors(checks, cr)
    sim.close()

    peak, peak_kind = peaks()
    bpp = bytes_per_px(C_CH, K_KER)
    step_s = ms / 1e3 / args.steps
    value = world * px * args.steps / (ms / 1e3)
    built = bytes_per_px_as_built(C_CH, K_KER, real) * px
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": warm, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": workload_config(world),
        # every step kernel against the roofline; the kernel with the
        # largest share of the step's device time on top
        "roofline": roofline_object(kms, N_GRID, C_CH, K_KER, peak, peak_kind, load_traffic(),
                                    real),
        # the step against HBM: first on the bytes the built passes move,
        # then on the survey's pass structure (which adds a forward column
        # pass of 8C B/px that this build fuses away)
        "step_hbm": {"kernel_spectra": "real (point-symmetric kernels)" if real else "complex",
                     "bytes_per_step_as_built": built,
                     "achieved_gbs_as_built": built / step_s / 1e9,
                     "frac_as_built": built / step_s / 1e9 / peak,
                     "bytes_per_step_algorithmic": bpp * px,
                     "frac_algorithmic": bpp * px / step_s / 1e9 / peak,
                     "peak_gbs": peak, "peak_source": peak_kind},
        "kernel_ms": {"row_r2c": kms[0], "col_conv": kms[1], "row_c2r_growth": kms[2],
                      "diffusion": kms[3]},
        "e2e": e2e,
        # per step one launch per phase (4) per channel (the graphs run the
        # channels on forked streams)
        "gpu_launches": 4 * C_CH * args.steps,
        "clocks": clocks,
        "autotune": tuned,
        "mass_drift": drift,
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
        line["step_error_vs_fp64"] = step_err
    if rank == 0 and world == 1 and not args.no_configs:
        # the other benchmark configurations, each with bounded repeats
        dev = torch.device("cuda", local)
        check = not args.no_cpu_baseline
        line["plain_1024"] = measure_plain_1024(dev, sampler, check=check)
        line["batched"] = measure_batched(dev, sampler, steps=500, warmup=3,
                                          autotune=not args.no_autotune, check=check)
        line["grad"] = measure_grad(dev, sampler, iters=10, warmup=3, check=check)
        line["search"] = measure_search(dev, sampler, iters=3, warmup=3, ncand=args.candidates,
                                        check=check)
        line["next_rows"] = measure_next_rows(dev, tuned["variants"] if tuned else [0, 0, 0, 0],
                                              check=check)
    sampler.stop()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def e2e_run(sim, cr, args, dist, world):
    """Per step through the public C ABI with host buffers: the upload of the
    state (f64, as upload_channel takes it) from pinned memory, one step, and
    the download of the f32 state to pinned memory.  The value is
    cg_step_host_async, which overlaps each step's upload with the previous
    step's compute and download (wall clock from the first call to
    cg_host_wait); `blocking` is the reference's call pattern
    upload_channel x C / iterate / download_all_channels, one step at a time."""
    import torch
    from cella_nova_gb300 import _abi
    px = cr.n * cr.n
    t_in = torch.empty((C_CH, px), dtype=torch.float64, pin_memory=True)
    t_out = torch.empty((C_CH * px,), dtype=torch.float32, pin_memory=True)
    host_in, host_out = t_in.numpy(), t_out.numpy()
    host_in[:] = cr.seed.reshape(C_CH, px)
    lib = sim._lib
    e2e_steps = max(3, min(args.steps, 50))

    def blocking_step():
        for c in range(C_CH):
            _abi.check(lib.cg_upload_channel(sim._h, c, _abi.dptr(host_in[c])))
        _abi.check(lib.cg_iterate(sim._h))
        _abi.check(lib.cg_download_channels(sim._h, _abi.fptr(host_out)))

    def pipelined_step():
        _abi.check(lib.cg_step_host_async(sim._h, _abi.dptr(host_in), _abi.fptr(host_out), 1))

    out = {}
    for name, one in (("blocking", blocking_step), ("pipelined", pipelined_step)):
        for _ in range(3):
            one()
        _abi.check(lib.cg_host_wait(sim._h))
        barrier(dist, world)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            one()
        _abi.check(lib.cg_host_wait(sim._h))
        out[name] = world * px * e2e_steps / max_over_ranks(time.perf_counter() - t0, dist, world)
    return {"value": out["pipelined"], "unit": UNIT,
            "h2d_bytes_per_step": C_CH * px * 8, "d2h_bytes_per_step": C_CH * px * 4,
            "steps": e2e_steps, "how": "cg_step_host_async per step (pinned f64 in, f32 out), "
                                       "then cg_host_wait",
            "blocking": {"value": out["blocking"], "unit": UNIT,
                         "how": "cg_upload_channel x C, cg_iterate, cg_download_channels"}}


def batched_creatures(device):
    """48 worlds at 1024^2 and 16 at 2048^2; C ~ U{1..4}, K = C^2 (all pairs),
    own mu/sigma/weights/ring kernels, temp ~ U[0.5, 2.0]."""
    from cella_nova_gb300.creature import make_creature
    rng = np.random.default_rng(64)
    sizes = [1024] * 48 + [2048] * 16
    out = []
    for i, n in enumerate(sizes):
        C = int(rng.integers(1, 5))
        out.append(make_creature(n, C, seed=10_000 + i, temp=float(rng.uniform(0.5, 2.0)),
                                 device=device))
    return out


def timed(stream, fn):
    """Device ms of fn()'s work on `stream` (CUDA events on that stream)."""
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1)


def measure_plain_1024(dev, sampler, steps=200, check=True):
    """The first benchmark configuration: one 1024^2 creature, C=3, K=9,
    ring radii U[12,30] px, `steps` graph steps (autotuned), with teacher-
    forced FP64 checks at three points of the run and the FP64 mass drift
    over all of it."""
    import torch
    from cella_nova_gb300 import GpuMaceLenia
    from cella_nova_gb300.creature import make_creature
    n = 1024
    cr = make_creature(n, 3, seed=1024, temp=1.0, device=dev)
    tb0 = time.perf_counter()
    sim = GpuMaceLenia.from_creature(cr)
    real = sim.kernels_real()
    m0 = sim.mass_f64()
    checks = {"step 1": sample_step(sim)}
    _, tune_ms = sim.autotune(reps=10)
    sim.run_steps(3)
    sim.synchronize()
    stream = torch.cuda.ExternalStream(sim.stream())
    tw0 = time.perf_counter()
    ms = timed(stream, lambda: sim.run_steps(steps))
    tw1 = time.perf_counter()
    checks[f"step {steps + 5}"] = sample_step(sim)
    sim.run_steps(steps - 1)
    checks[f"step {2 * steps + 5}"] = sample_step(sim)
    m1 = sim.mass_f64()
    tb1 = time.perf_counter()
    variants = sim.variants()
    layout = sim.graph_layout()
    sim.close()
    px = n * n
    out = {"metric": "cell-updates/s (DiffusionLenia fwd step, 1024^2, C=3, K=9)",
           "value": px * steps / (ms / 1e3), "unit": UNIT, "steps": steps,
           "ms_per_step": ms / steps, "variants": variants, "graph_layout": layout,
           "autotune_ms": [[round(float(t), 4) for t in row] for row in tune_ms],
           "kernel_spectra": "real (point-symmetric kernels)" if real else "complex",
           "hbm_frac_as_built": bytes_per_px_as_built(3, 9, real) * px / (ms / 1e3 / steps) / 1e9
           / peaks()[0],
           "mass_drift": {"steps": 2 * steps + 6, "max_rel": float(np.abs(m1 / m0 - 1).max()),
                          "reduction": "FP64 on the GPU"},
           "clocks": sampler.summary(tw0, tw1, (tb0, tb1, "autotune, warm-up, timed and "
                                                            "checked steps")),
           "l2": "no flush: each step streams ~0.2 GB (> 129 MB L2)"}
    if check:
        out["step_error_vs_fp64"] = step_errors(checks, cr)
    return out


def measure_next_rows(dev, variants, reps=50, check=True):
    """The survey's "next" rows on the 2048^2, C=3, K=9 creature, each with a
    figure and a parity check:
    - render: a rendering step against a plain step, the standalone render
      kernel, the RGB24 download, and frame streaming to a
      file descriptor (the video loop, main.rs:239-303); render words against
      the FP32 restatement of render_main (compute_1024.wgsl:428-443);
    - kernel builder: K ring kernels built and transformed on the GPU against
      the host generator (numpy ring kernels and FFT in FP64, what
      generate_kernel_json.py does), two kernels timed and scaled to K; a step
      with the built spectra against one with the host spectra;
    - binary seed: load time of a 1024^2, C=3 seed as JSON and as its binary
      twin, and the two loads compared value for value."""
    import tempfile
    import torch
    from cella_nova_gb300 import GpuMaceLenia
    from cella_nova_gb300.creature import (make_creature, ring_kernel, write_seed_bin,
                                           write_seed_json)
    from cella_nova_gb300.orchestrator import creature_ring_specs, load_config
    n, px = N_GRID, N_GRID * N_GRID
    cr = make_creature(n, C_CH, seed=2048, temp=1.0, device=dev)
    out = {}
    with GpuMaceLenia.from_creature(cr) as sim:
        sim.set_variants(variants)
        stream = torch.cuda.ExternalStream(sim.stream())
        for _ in range(3):
            sim.iterate()
            sim.iterate_and_render()
            sim.render()
        sim.synchronize()
        plain = timed(stream, lambda: [sim.iterate() for _ in range(reps)]) / reps
        fused = timed(stream, lambda: [sim.iterate_and_render() for _ in range(reps)]) / reps
        alone = timed(stream, lambda: [sim.render() for _ in range(reps)]) / reps
        t0 = time.perf_counter()
        for _ in range(5):
            rgb = sim.download_render()
        dl_s = (time.perf_counter() - t0) / 5
        nframes = 20
        with open(os.devnull, "wb") as f:
            t0 = time.perf_counter()
            sim.stream_frames(f.fileno(), nframes, 1)
            fr_s = time.perf_counter() - t0
        render = {"step_ms": plain, "step_with_render_ms": fused,
                  "render_cost_ms": fused - plain,
                  "render_how": "iterate_and_render: the diffusion kernels also write level "
                                "bytes, then one kernel packs them into 0x00RRGGBB words",
                  "render_kernel_ms": alone,
                  "render_kernel_gbs": (C_CH * 4 + 4) * px / (alone / 1e3) / 1e9,
                  "download_rgb24_ms": dl_s * 1e3,
                  "frames_per_s": nframes / fr_s,
                  "frames": f"{nframes} RGB24 frames of {n}^2 to /dev/null, one step each "
                            "(cg_stream_frames)"}
        if check:
            from oracle import oracle as O
            sim.iterate_and_render()
            words = sim.download_render_packed()
            render["words_equal_oracle"] = bool(np.array_equal(words, O.render_np(sim.state())))
            render["rgb24_equal_oracle"] = bool(np.array_equal(sim.download_render(),
                                                               O.rgb24_np(words)))
        out["render"] = render

        # kernel builder
        specs, w = creature_ring_specs(cr)
        wd = torch.tensor(w, device=dev)
        torch.cuda.synchronize()
        x = sim.state()
        sim.build_ring_kernels(specs, wd.data_ptr())   # warm-up (re-captures the graphs once)
        sim.synchronize()
        build = timed(stream, lambda: [sim.build_ring_kernels(specs, wd.data_ptr())
                                       for _ in range(10)]) / 10
        t0 = time.perf_counter()
        nk = 2
        for k in range(nk):
            np.fft.fft2(ring_kernel(n, cr.ring_radius[k], cr.ring_weights[k]))
        host_s = (time.perf_counter() - t0) / nk * cr.K
        builder = {"kernels": cr.K, "gpu_ms": build, "host_generator_ms": host_s * 1e3,
                   "host_how": f"numpy ring kernel + FP64 fft2 per kernel, {nk} of {cr.K} "
                               f"timed and scaled to {cr.K}, one host thread"}
        # one step from the same state with the built spectra, then with the
        # host spectra (cg_set_kernel)
        for c in range(C_CH):
            sim.upload_channel_f32(x[c], c)
        sim.iterate()
        y_built = sim.state()
        for k in range(cr.K):
            sim.set_kernel(cr.kspec[k], k)
        for c in range(C_CH):
            sim.upload_channel_f32(x[c], c)
        sim.iterate()
        builder["step_max_abs_diff_vs_host_spectra"] = float(np.abs(y_built - sim.state()).max())
        out["kernel_builder"] = builder

    # binary seed against JSON
    seed_cr = make_creature(1024, 3, seed=1024)
    with tempfile.TemporaryDirectory() as d:
        js, bs = os.path.join(d, "s.json"), os.path.join(d, "s.bin")
        write_seed_json(js, seed_cr)
        write_seed_bin(bs, seed_cr)
        times = {}
        cfgs = {}
        for name, path in (("json", js), ("binary", bs)):
            best = None
            for _ in range(2):
                t0 = time.perf_counter()
                cfgs[name] = load_config(path)
                dt = time.perf_counter() - t0
                best = dt if best is None else min(best, dt)
            times[name] = best
        same = all(np.array_equal(np.asarray(cfgs["json"][k]), np.asarray(cfgs["binary"][k]))
                   for k in cfgs["json"])
        out["binary_seed"] = {"seed": "1024^2, C=3", "json_load_ms": times["json"] * 1e3,
                              "binary_load_ms": times["binary"] * 1e3,
                              "json_bytes": os.path.getsize(js), "binary_bytes": os.path.getsize(bs),
                              "same_values": bool(same)}
    return out


def measure_batched(dev, sampler, steps=500, warmup=3, autotune=True, check=True,
                    plain_steps=20):
    """Batched forward: every world advanced by one persistent launch per
    phase per grid side, one CUDA graph per step; against the plain
    single-world path on the same worlds, one world at a time."""
    import torch
    from cella_nova_gb300 import GpuMaceLenia, GpuMaceLeniaBatch
    t0 = time.perf_counter()
    crs = batched_creatures(dev)
    gen_s = time.perf_counter() - t0
    cells = sum(cr.n * cr.n for cr in crs)
    b = GpuMaceLeniaBatch(crs)
    m0 = [b.mass_f64(i) for i in range(len(crs))]
    tuned = None
    if autotune:
        tuned = {str(k): {"variants": v[0], "ms": np.round(v[1], 4).tolist()}
                 for k, v in b.autotune(reps=5).items()}
    stream = torch.cuda.ExternalStream(b.stream())
    b.run_steps(max(warmup, 3))
    b.synchronize()
    tw0 = time.perf_counter()
    ms = timed(stream, lambda: b.run_steps(steps))
    tw1 = time.perf_counter()
    clocks = sampler.summary(tw0, tw1)
    phase_ms = b.profile(min(max(steps, 4), 32))
    items, grid = b.info()
    modes = {str(side): b.mode(side) for side in sorted({cr.n for cr in crs})}
    # one teacher-forced step of one world of each grid side against FP64
    checks = {}
    if check:
        for side in sorted({cr.n for cr in crs}):
            w = next(i for i, cr in enumerate(crs) if cr.n == side)
            x = b.state(w)
            b.run_steps(1)
            checks[f"world {w} ({side}^2, C={crs[w].C})"] = oracle_step_error(x, b.state(w),
                                                                              crs[w])
    drift = max(float(np.abs(b.mass_f64(i) / m0[i] - 1).max()) for i in range(len(crs)))
    b.close()
    # the plain single-world path on the same worlds, one world at a time
    # (each world autotuned like the batch)
    plain_s = 0.0
    for cr in crs:
        s = GpuMaceLenia.from_creature(cr)
        if autotune:
            s.autotune(reps=3)
        s.run_steps(2)
        s.synchronize()
        plain_s += timed(torch.cuda.ExternalStream(s.stream()),
                         lambda: s.run_steps(plain_steps)) / 1e3 / plain_steps
        s.close()
    out = {
        "metric": "cell-updates/s (batched fwd: 48x1024^2 + 16x2048^2, C in 1..4, K=C^2)",
        "value": cells * steps / (ms / 1e3), "unit": UNIT, "steps": steps,
        "warmup": max(warmup, 3), "ms_per_step": ms / steps,
        "config": {"workload": "64 worlds (48 at 1024^2, 16 at 2048^2), channels U{1..4}, "
                               "kernels = all pairs, temp U[0.5,2]; one persistent launch per "
                               "phase per grid side, one CUDA graph per step",
                   "worlds": len(crs), "cells_per_step": cells,
                   "channels": [cr.C for cr in crs]},
        "plain_loop": {"value": cells / plain_s, "unit": UNIT, "ms_per_step": 1e3 * plain_s,
                       "how": f"same worlds, the single-world graph path one world at a time, "
                              f"{plain_steps} steps each"},
        "batched_over_plain": (1e3 * plain_s) / (ms / steps),
        "phase_ms": {"row_r2c": phase_ms[0], "col_conv": phase_ms[1],
                     "row_c2r_growth": phase_ms[2], "diffusion": phase_ms[3]},
        "work_items": items, "persistent_grid": grid, "autotune": tuned,
        # per grid side: 0 = one persistent launch per phase over its worlds,
        # 1 = each world's own step kernels as parallel graph branches
        "modes": modes,
        "mass_drift": {"max_rel": drift, "steps": max(warmup, 3) + steps + 32 + len(checks),
                       "reduction": "FP64 on the GPU, every world"},
        # mode 0: one persistent launch per phase per grid side; mode 1: per
        # world one launch per phase and channel
        "gpu_launches": steps * sum(4 if modes[str(side)] == 0 else
                                    4 * sum(cr.C for cr in crs if cr.n == side)
                                    for side in {cr.n for cr in crs}),
        "clocks": clocks,
        "setup_s": {"generate": gen_s},
    }
    if checks:
        out["step_error_vs_fp64"] = {"max_abs": max(checks.values()), "bar": 1e-5,
                                     "worlds": checks,
                                     "how": "teacher-forced batched step of one world per grid "
                                            "side against the FP64 oracle"}
    return out


def run_batched(args):
    import torch
    world, rank, local, dist = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    sampler = ClockSampler(local)
    sampler.start()
    out = measure_batched(torch.device("cuda", local), sampler, steps=args.steps,
                          warmup=args.warmup, autotune=not args.no_autotune,
                          check=not args.no_cpu_baseline)
    sampler.stop()
    ms = max_over_ranks(out["ms_per_step"] * out["steps"], dist, world)
    cells = out["config"]["cells_per_step"]
    line = dict(out, value=world * cells * out["steps"] / (ms / 1e3), n_gpus=world,
                ms_per_step=ms / out["steps"], higher_is_better=True, scaling="weak",
                vs_baseline=None, dtype="f32", data="synthetic")
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def measure_grad(dev, sampler, iters=20, warmup=3, check=True):
    """Differentiable unroll: one 1024^2 creature, C=3, K=9, T=64 steps,
    checkpoints every 8; loss = MSE(x_T, seed shifted by (+16, +8) px);
    gradients for the seed, mu, sigma, weights and ring weights through the
    adjoint kernels.  fwd+bwd cell-updates/s = n^2 T / (forward + backward).
    The gradient check runs the same construction on the 128^2 instance
    (T=64, checkpoints every 8) against FP64 autograd."""
    import torch
    from cella_nova_gb300.autograd import DiffusionLeniaGPU
    from cella_nova_gb300.creature import make_creature
    n, C, T, every = 1024, 3, 64, 8
    cr = make_creature(n, C, seed=1024, temp=1.0, device=dev)
    target = torch.tensor(np.roll(cr.seed, (8, 16), axis=(1, 2)), dtype=torch.float32,
                          device=dev)
    m = DiffusionLeniaGPU(cr)

    def iteration():
        m.zero_grad(set_to_none=True)
        xT = m(T, every)
        loss = torch.mean((xT - target) ** 2)
        loss.backward()
        return loss, xT

    tb0 = time.perf_counter()
    for _ in range(max(warmup, 3)):
        iteration()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    f_ms = b_ms = 0.0
    tw0 = time.perf_counter()
    for _ in range(iters):
        m.zero_grad(set_to_none=True)
        ev[0].record()
        xT = m(T, every)
        loss = torch.mean((xT - target) ** 2)
        ev[1].record()
        loss.backward()
        ev[2].record()
        ev[2].synchronize()
        f_ms += ev[0].elapsed_time(ev[1])
        b_ms += ev[1].elapsed_time(ev[2])
    tw1 = time.perf_counter()
    f_ms, b_ms = f_ms / iters, b_ms / iters
    # mass of x_T against the seed's, FP64 on the GPU
    mT = xT.detach().double().sum(dim=(1, 2))
    m0 = m.seed.detach().double().sum(dim=(1, 2))
    drift = float((mT / m0 - 1).abs().max())
    out = {
        "metric": "cell-updates/s (fwd+bwd, differentiable unroll 1024^2, C=3, K=9, T=64, "
                  "checkpoints every 8)",
        "value": n * n * T / ((f_ms + b_ms) / 1e3), "unit": UNIT, "steps": iters,
        "warmup": max(warmup, 3), "ms_per_step": f_ms + b_ms,
        "config": {"workload": "1 creature 1024^2, 3 channels, 9 kernels, T=64, checkpoint every "
                               "8 (backward recomputes each segment), loss MSE vs seed shifted "
                               "(+16,+8) px; grads: seed, mu, sigma, weights, ring weights",
                   "step_unit": "one forward+backward iteration of the unroll"},
        "forward_ms": f_ms, "backward_ms": b_ms,
        "forward_cell_updates_per_s": n * n * T / (f_ms / 1e3),
        # forward 4 per step; the backward re-runs each segment (4 per step,
        # 3 for a segment's last) and runs 5 adjoint kernels per step; kernel
        # build 4 + parameter fold 1 in each direction; 2 final kernel-gradient
        # and 2 ring-gradient launches
        "gpu_launches": 13 * T - (T + every - 1) // every + 14,
        "loss": float(loss.detach()), "mass_drift": {"max_rel": drift, "steps": T,
                                                     "reduction": "FP64 on the GPU"},
        "clocks": sampler.summary(tw0, tw1, (tb0, tw1, "warm-up and timed iterations")),
    }
    del m
    if check:
        out["grad_check"] = grad_check_128(dev)
    return out


def grad_check_128(dev, T=64, every=8):
    """The GPU gradients of the differentiable unroll on the 128^2 instance
    (C=3, K=9, T=64, checkpoints every 8) against FP64 autograd of the step
    (oracle/autograd_ref.py, itself pinned to the reference model's autograd
    and to finite differences), relative to each gradient's largest
    component."""
    import torch
    from cella_nova_gb300.autograd import DiffusionLeniaGPU
    from cella_nova_gb300.creature import make_creature
    from oracle import autograd_ref as AR
    n = 128
    cr = make_creature(n, 3, seed=128, radius=(n / 16, n / 6), seed_box=n // 2, temp=1.0)
    target = AR.shifted_target(cr.seed)
    t0 = time.perf_counter()
    ref = AR.gradients(cr, T, target)
    el = time.perf_counter() - t0
    m = DiffusionLeniaGPU(cr)
    xT = m(T, every)
    loss = torch.mean((xT - torch.tensor(target, dtype=torch.float32, device=dev)) ** 2)
    loss.backward()

    def rel(a, b):
        a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
        return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))

    err = {"seed": rel(m.seed.grad.cpu(), ref["seed"]), "mu": rel(m.mu.grad.cpu(), ref["mu"]),
           "sigma": rel(m.sigma.grad.cpu(), ref["sigma"]),
           "weights": rel(m.weights.grad.cpu(), ref["weights"]),
           "ring_weights": rel(np.concatenate([b.grad.cpu().numpy() for b in m.ring_weights]),
                               np.concatenate(ref["ring_weights"]))}
    return {"instance": f"{n}^2, C=3, K=9, T={T}, checkpoints every {every}",
            "max_rel_error": err, "loss_rel_error": abs(float(loss.detach()) / ref["loss"] - 1),
            "oracle_s": el}


def run_grad(args):
    import torch
    world, rank, local, dist = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    sampler = ClockSampler(local)
    sampler.start()
    out = measure_grad(torch.device("cuda", local), sampler, iters=max(1, min(args.steps, 20)),
                       warmup=args.warmup, check=not args.no_cpu_baseline and world == 1)
    sampler.stop()
    tot = max_over_ranks(out["ms_per_step"], dist, world)
    line = dict(out, value=world * 1024 * 1024 * 64 / (tot / 1e3), n_gpus=world,
                ms_per_step=tot, higher_is_better=True, scaling="weak", vs_baseline=None,
                dtype="f32", data="synthetic")
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def measure_search(dev, sampler, iters=3, warmup=3, ncand=32, check=True):
    """Batched gradient search: `ncand` candidates at 1024^2, C=3, K=9,
    T=128, checkpoints every 16, MSE to the seed shifted by (+16, +8) px,
    Adam on the seed, mu, sigma, weights and ring weights; every iteration of
    all candidates is one CUDA graph (Adam included).  fwd+bwd cell-updates/s
    = candidates * n^2 * T / iteration time, against the plain per-creature
    loop over every candidate (torch autograd over the same kernels +
    torch.optim.Adam, one candidate at a time)."""
    import torch
    from cella_nova_gb300 import _abi
    from cella_nova_gb300.autograd import DiffusionLeniaGPU
    from cella_nova_gb300.creature import make_creature
    from cella_nova_gb300.search import AdamConfig, GradientSearch
    n, C, T, every = 1024, 3, 128, 16
    t0 = time.perf_counter()
    crs = [make_creature(n, C, seed=5000 + i, temp=1.0, device=dev) for i in range(ncand)]
    tgs = [np.roll(cr.seed, (8, 16), axis=(1, 2)) for cr in crs]
    gen_s = time.perf_counter() - t0
    adam = AdamConfig(lr_seed=1e-3, lr_params=1e-3, lr_rings=1e-2)
    gs = GradientSearch(crs, tgs, T=T, every=every, adam=adam, n_streams=4)
    warm = max(warmup, 3)
    gs.run(1)                         # the first iteration eagerly (allocates scratch)
    loss_first = float(np.mean(gs.losses()))
    gs.run(warm - 1)                  # capture, then replays
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    tw0 = time.perf_counter()
    e0.record()
    gs.run(iters)
    e1.record()
    e1.synchronize()
    tw1 = time.perf_counter()
    ms = e0.elapsed_time(e1) / iters
    clocks = sampler.summary(tw0, tw1)
    losses = gs.losses()
    # mass of x_T of the last iteration against the x_0 it was unrolled from
    # (the first checkpoint), FP64 on the GPU
    lib = _abi.load()
    drift = 0.0
    m0 = torch.zeros(C, dtype=torch.float64, device=dev)
    m1 = torch.zeros_like(m0)
    torch.cuda.synchronize()
    for c in gs.cands:
        _abi.check(lib.cg_mass_f64_noalloc(ctypes.c_void_p(c.ckpt.data_ptr()), n, C,
                                           ctypes.c_void_p(m0.data_ptr()), None))
        _abi.check(lib.cg_mass_f64_noalloc(ctypes.c_void_p(c.xT.data_ptr()), n, C,
                                           ctypes.c_void_p(m1.data_ptr()), None))
        torch.cuda.synchronize()
        drift = max(drift, float((m1 / m0 - 1).abs().max()))
    gs.close()

    # plain per-creature loop over every candidate: torch autograd over the
    # same adjoint kernels and torch.optim.Adam, one candidate at a time (no
    # graphs); each candidate's first iteration is its warm-up
    tgt = [torch.tensor(tg, dtype=torch.float32, device=dev) for tg in tgs]
    plain_ms = 0.0
    for i in range(ncand):
        mdl = DiffusionLeniaGPU(crs[i])
        opt = torch.optim.Adam([{"params": [mdl.seed], "lr": adam.lr_seed},
                                {"params": [mdl.mu, mdl.sigma, mdl.weights],
                                 "lr": adam.lr_params},
                                {"params": list(mdl.ring_weights), "lr": adam.lr_rings}])

        def plain_iteration():
            opt.zero_grad(set_to_none=True)
            loss = torch.mean((mdl(T, every) - tgt[i]) ** 2)
            loss.backward()
            opt.step()

        plain_iteration()
        torch.cuda.synchronize()
        plain_ms += timed(torch.cuda.current_stream(), plain_iteration)
        del mdl, opt
    cells = ncand * n * n * T
    out = {
        "metric": "cell-updates/s (batched gradient search fwd+bwd: 32 x 1024^2, C=3, K=9, "
                  "T=128, checkpoints every 16, in-graph Adam)",
        "value": cells / (ms / 1e3), "unit": UNIT, "steps": iters, "warmup": warm,
        "ms_per_step": ms,
        "config": {"workload": f"{ncand} candidates 1024^2, 3 channels, 9 kernels (all pairs), "
                               "ring kernels built on the GPU each iteration, T=128, checkpoint "
                               "every 16, loss MSE vs seed shifted (+16,+8) px, Adam on seed, "
                               "mu, sigma, weights, ring weights; one CUDA graph per iteration "
                               "over 4 streams",
                   "step_unit": "one iteration (forward, backward, Adam) of every candidate",
                   "candidates": ncand},
        "plain_loop": {"value": cells / (plain_ms / 1e3), "unit": UNIT, "ms_per_step": plain_ms,
                       "how": f"torch autograd + torch.optim.Adam, one candidate at a time, "
                              f"all {ncand} candidates timed (one iteration each after one "
                              f"warm-up iteration)"},
        "batched_over_plain": plain_ms / ms,
        "loss_mean": float(np.mean(losses)),
        "loss_mean_first_iteration": loss_first,
        "iterations_total": warm + iters,
        "mass_drift": {"max_rel": drift, "steps": T, "reduction": "FP64 on the GPU"},
        # per candidate and iteration: builder 4, parameter fold 1, forward 4
        # per step, MSE 2, segment recompute 4 per step (3 for a segment's
        # last), backward 5 per step, kernel gradient 2, ring gradient 2, Adam
        # 3; plus the step counter once per iteration
        "gpu_launches": iters * (ncand * (13 * T - (T + every - 1) // every + 14) + 1),
        "clocks": clocks,
        "setup_s": {"generate": gen_s},
    }
    if check:
        out["cpu_baseline"], out["grad_check"] = search_cpu_check()
    return out


def run_search(args):
    import torch
    world, rank, local, dist = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    sampler = ClockSampler(local)
    sampler.start()
    out = measure_search(torch.device("cuda", local), sampler, iters=max(1, args.steps),
                         warmup=args.warmup, ncand=args.candidates,
                         check=not args.no_cpu_baseline and world == 1)
    sampler.stop()
    ms = max_over_ranks(out["ms_per_step"], dist, world)
    cells = out["config"]["candidates"] * 1024 * 1024 * 128
    line = dict(out, value=world * cells / (ms / 1e3), n_gpus=world, ms_per_step=ms,
                higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f32",
                data="synthetic")
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def search_cpu_check():
    """CPU leg: the FP64 autograd oracle (torch, float64, all host threads)
    on a bounded sample -- one 128^2 candidate, C=3, K=9, T=16, checkpoints
    every 4 -- timed as fwd+bwd cell-updates/s, and used to check
    the GPU search's gradients on the same instance."""
    import torch
    from cella_nova_gb300.creature import make_creature
    from cella_nova_gb300.search import GradientSearch
    from oracle import autograd_ref as AR
    n, C, T, every = 128, 3, 16, 4
    cr = make_creature(n, C, seed=777, temp=1.0, radius=(6, 20), seed_box=64)
    tg = AR.shifted_target(cr.seed)
    t0 = time.perf_counter()
    ref = AR.gradients(cr, T, tg, ring=True)
    el = time.perf_counter() - t0
    with GradientSearch([cr], [tg], T=T, every=every, n_streams=1) as gs:
        gs.run_eager(1)
        got = gs.gradients(0)

    def rel(a, b):
        a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
        return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))

    err = {k: rel(got[k], ref[k]) for k in ("seed", "mu", "sigma", "weights")}
    err["ring_weights"] = rel(np.concatenate([got["ring_weights"][k, :len(b)]
                                              for k, b in enumerate(ref["ring_weights"])]),
                              np.concatenate(ref["ring_weights"]))
    cpu = {"value": n * n * T / el, "unit": UNIT, "cores": torch.get_num_threads(),
           "kind": "port",
           "sample": f"FP64 torch autograd of the step (oracle/autograd_ref.py), one {n}^2 "
                     f"C={C} K=9 candidate, T={T}, fwd+bwd, {el:.1f} s"}
    check = {"instance": f"{n}^2, C={C}, K=9, T={T}", "max_rel_error": err,
             "loss_rel_error": abs(got["loss"] / ref["loss"] - 1)}
    return cpu, check


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # default: 4000 steps for the plain 2048^2 step (a timed region near one
    # second, ~10 clock samples), 500 for the batched forward, 20 iterations
    # of the differentiable unroll
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--variants", default=None,
                    help="fixed CTA-shape variants r2c,col,c2r,diffusion (skips the autotuner)")
    ap.add_argument("--config", default="plain", choices=["plain", "batched", "grad", "search"])
    ap.add_argument("--candidates", type=int, default=32)
    ap.add_argument("--no-configs", action="store_true",
                    help="default run: skip the sub-objects of the other configurations")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = {"plain": 4000, "batched": 500, "grad": 20, "search": 3}[args.config]
        if args.impl == "reference":
            args.steps = 1000
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "batched":
        return run_batched(args)
    if args.config == "grad":
        return run_grad(args)
    if args.config == "search":
        return run_search(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
