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


def bytes_per_px_as_built(C, K):
    """The same for the passes this library runs: the forward column FFT is
    fused into the column convolution, so its 8C never reach HBM (row pass 8C,
    column pass 4C + 8K, inverse row pass 4K + 4C, diffusion 12C)."""
    return 28 * C + 12 * K


def col_conv_bytes_per_px(C, K):
    """k_col_conv: read the row spectra once (4C), read each kernel's half
    spectrum and write its column-inverted product (8K)."""
    return 4 * C + 8 * K


# Algorithmic bytes per grid point of each step kernel, in the order of
# profile_kernels' split (row_r2c, col_conv, row_c2r_growth, diffusion).
KERNEL_NAMES = ("k_row_r2c", "k_col_conv", "k_row_c2r_growth", "k_diffusion")


def kernel_bytes_per_px(C, K):
    return (8 * C,                       # read the state, write the row spectra
            col_conv_bytes_per_px(C, K),
            4 * K + 4 * C,               # read each U, write A
            12 * C)                      # read A and the state, write the new state


def roofline_object(kms, n, C, K, peak, peak_kind, traffic=None):
    """The `roofline` object of the bench line: every step kernel's
    algorithmic bytes per launch (kernel_bytes_per_px x n^2) over its
    measured duration (kms, ms per step, in KERNEL_NAMES order) against the
    peak, and the kernel with the largest device time reported on top.
    `traffic` maps "<kernel>_<n>" to an ncu capture's DRAM bytes per launch."""
    traffic = traffic or {}
    px = n * n
    per_kernel = []
    for name, b, t in zip(KERNEL_NAMES, kernel_bytes_per_px(C, K), kms):
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
    """nvidia-smi clocks and throttle reasons sampled every 100 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
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
        for line in self.proc.stdout:
            self.rows.append((time.perf_counter(), [x.strip() for x in line.split(",")]))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self, t0=None, t1=None):
        rows = [r for t, r in self.rows if (t0 is None or t >= t0) and (t1 is None or t <= t1)]
        if not rows:
            rows = [r for _, r in self.rows]
        if not rows:
            why = ("nvidia-smi printed no sample (the run may be shorter than its start-up)"
                   if self.proc else "nvidia-smi unavailable")
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0,
                    "note": why}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if len(r) > 5 + i and r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


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


def step_error_vs_fp64(sim, cr):
    """Checker beside the CPU baseline: one GPU step from the GPU's current
    state against the FP64 oracle's step from the same state (numpy FP64
    twin of example.rs), max-abs over the whole 2048^2 grid."""
    from oracle import oracle as O
    x = sim.state()
    sim.iterate()
    y = sim.state()
    ref, _, _ = O.step_np(x.astype(np.float64), cr.kspec.astype(np.complex128), cr.c0, cr.c1,
                          cr.mu.astype(np.float64), cr.sigma.astype(np.float64),
                          cr.weights.astype(np.float64), cr.temp)
    return float(np.abs(y - ref).max())


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
    for _ in range(min(args.warmup, 1)):
        st, _, _ = O.step_c(st, ks, *a, dtype=np.float32, faithful=True, nthreads=nthreads)
    budget = 150.0
    done, t0 = 0, time.perf_counter()
    while done < args.steps:
        st, _, _ = O.step_c(st, ks, *a, dtype=np.float32, faithful=True, nthreads=nthreads)
        done += 1
        if time.perf_counter() - t0 > budget:
            break
    el = time.perf_counter() - t0
    value = N_GRID * N_GRID * done / el
    sample = (f"{done} of {args.steps} requested steps (150 s budget), f32 C port of "
              f"example.rs, OpenMP {nthreads} threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": done, "warmup": min(args.warmup, 1),
        "ms_per_step": 1e3 * el / done, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "n": N_GRID, "channels": C_CH, "kernels": K_KER,
                   "device": "host CPU"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


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

    cr = make_creature(N_GRID, C_CH, seed=2048 + rank, temp=1.0)
    sim = GpuMaceLenia.from_creature(cr)
    px = N_GRID * N_GRID
    tuned = None
    if args.variants:
        sim.set_variants([int(v) for v in args.variants.split(",")])
        tuned = {"variants": sim.variants(), "ms": None, "how": "--variants"}
    elif not args.no_autotune:
        chosen, tms = sim.autotune(reps=10)
        tuned = {"variants": chosen, "ms": np.round(tms, 4).tolist()}
    stream = torch.cuda.ExternalStream(sim.stream())
    sampler = ClockSampler(local)
    sampler.start()

    mass0 = sim.mass_f64()
    # warm-up, then K timed graph launches between barriers + syncs
    sim.run_steps(max(args.warmup, 3))
    sim.synchronize()
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
    clocks = sampler.summary(t_wall0, t_wall1)

    mass1 = sim.mass_f64()
    drift = {"steps": max(args.warmup, 3) + args.steps,
             "max_rel": float(np.abs(mass1 / mass0 - 1).max()), "reduction": "FP64 on the GPU"}

    # per-kernel device time with events between kernels (same stream)
    prof_steps = min(max(args.steps, 8), 256)
    kms = sim.profile_kernels(prof_steps)
    sim.synchronize()

    # end to end through the public API with host buffers: per step, upload
    # the state (f64, as upload_channel takes it) from pinned memory, step,
    # download the f32 state
    e2e = None
    if not args.no_e2e:
        e2e = e2e_run(sim, cr, args, dist, world)
    sampler.stop()

    cpu = step_err = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(cr)
        step_err = step_error_vs_fp64(sim, cr)

    peak, peak_kind = peaks()
    bpp = bytes_per_px(C_CH, K_KER)
    step_s = ms / 1e3 / args.steps
    value = world * px * args.steps / (ms / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "n": N_GRID, "channels": C_CH, "kernels": K_KER,
                   "parallelism": f"replicas x{world}",
                   "l2": "no flush: each step streams ~0.75 GB (> 129 MB L2)"},
        # every step kernel against the roofline; the kernel with the
        # largest share of the step's device time on top
        "roofline": roofline_object(kms, N_GRID, C_CH, K_KER, peak, peak_kind, load_traffic()),
        "step_hbm": {"bytes_per_step": bpp * px, "achieved_gbs": bpp * px / step_s / 1e9,
                     "frac": bpp * px / step_s / 1e9 / peak, "peak_source": peak_kind,
                     "bytes_per_step_as_built": bytes_per_px_as_built(C_CH, K_KER) * px,
                     "frac_as_built": bytes_per_px_as_built(C_CH, K_KER) * px / step_s / 1e9 / peak},
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
        line["step_error_vs_fp64"] = {"max_abs": step_err, "bar": 1e-5,
                                      "how": "one step from the GPU state after the timed run, "
                                             "against the FP64 oracle from the same state"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    sim.close()
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


def run_batched(args):
    """Batched forward: every world advanced by one persistent launch per
    phase, one CUDA graph per step; against the plain per-world path."""
    import torch
    world, rank, local, dist = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    from cella_nova_gb300 import GpuMaceLenia, GpuMaceLeniaBatch
    t0 = time.perf_counter()
    crs = batched_creatures(torch.device("cuda", local))
    gen_s = time.perf_counter() - t0
    cells = sum(cr.n * cr.n for cr in crs)
    b = GpuMaceLeniaBatch(crs)
    tuned = None
    if not args.no_autotune:
        tuned = {str(k): {"variants": v[0], "ms": np.round(v[1], 4).tolist()}
                 for k, v in b.autotune(reps=5).items()}
    stream = torch.cuda.ExternalStream(b.stream())
    sampler = ClockSampler(local)
    sampler.start()
    b.run_steps(max(args.warmup, 3))
    b.synchronize()
    barrier(dist, world)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    tw0 = time.perf_counter()
    e0.record(stream)
    b.run_steps(args.steps)
    e1.record(stream)
    e1.synchronize()
    tw1 = time.perf_counter()
    ms = max_over_ranks(e0.elapsed_time(e1), dist, world)
    clocks = sampler.summary(tw0, tw1)
    phase_ms = b.profile(min(max(args.steps, 4), 32))
    items, grid = b.info()
    b.close()
    # the plain single-world path on the same worlds, one world at a time
    # (each world autotuned like the batch)
    plain_steps = max(3, min(args.steps, 20))
    plain_s = 0.0
    for cr in crs:
        s = GpuMaceLenia.from_creature(cr)
        if not args.no_autotune:
            s.autotune(reps=3)
        s.run_steps(2)
        s.synchronize()
        st = torch.cuda.ExternalStream(s.stream())
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(st)
        s.run_steps(plain_steps)
        a1.record(st)
        a1.synchronize()
        plain_s += a0.elapsed_time(a1) / 1e3 / plain_steps
        s.close()
    sampler.stop()
    value = world * cells * args.steps / (ms / 1e3)
    line = {
        "metric": "cell-updates/s (batched fwd: 48x1024^2 + 16x2048^2, C in 1..4, K=C^2)",
        "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "64 worlds (48 at 1024^2, 16 at 2048^2), channels U{1..4}, "
                               "kernels = all pairs, temp U[0.5,2]; one persistent launch per "
                               "phase, one CUDA graph per step",
                   "worlds": len(crs), "cells_per_step": cells,
                   "channels": [cr.C for cr in crs]},
        "plain_loop": {"value": world * cells / plain_s, "unit": UNIT,
                       "ms_per_step": 1e3 * plain_s,
                       "how": "same worlds, the single-world graph path one world at a time"},
        "batched_over_plain": (cells / (ms / 1e3 / args.steps)) / (cells / plain_s),
        "phase_ms": {"row_r2c": phase_ms[0], "col_conv": phase_ms[1],
                     "row_c2r_growth": phase_ms[2], "diffusion": phase_ms[3]},
        "work_items": items, "persistent_grid": grid, "autotune": tuned,
        # one persistent launch per phase per grid size
        "gpu_launches": 4 * len({cr.n for cr in crs}) * args.steps, "clocks": clocks,
        "setup_s": {"generate": gen_s},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_grad(args):
    """Differentiable unroll: one 1024^2 creature, C=3, K=9, T=64 steps,
    checkpoints every 8; loss = MSE(x_T, seed shifted by (+16, +8) px);
    gradients for the seed, mu, sigma, weights and ring weights through the
    adjoint kernels.  fwd+bwd cell-updates/s = n^2 T / (forward + backward)."""
    import torch
    world, rank, local, dist = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    from cella_nova_gb300.autograd import DiffusionLeniaGPU
    from cella_nova_gb300.creature import make_creature
    n, C, T, every = 1024, 3, 64, 8
    cr = make_creature(n, C, seed=1024 + rank, temp=1.0, device=torch.device("cuda", local))
    target = torch.tensor(np.roll(cr.seed, (8, 16), axis=(1, 2)), dtype=torch.float32,
                          device="cuda")
    m = DiffusionLeniaGPU(cr)

    def iteration():
        m.zero_grad(set_to_none=True)
        xT = m(T, every)
        loss = torch.mean((xT - target) ** 2)
        loss.backward()
        return loss

    for _ in range(max(args.warmup, 3)):
        iteration()
    torch.cuda.synchronize()
    barrier(dist, world)
    iters = max(1, min(args.steps, 20))
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    f_ms = b_ms = 0.0
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
    f_ms, b_ms = f_ms / iters, b_ms / iters
    tot = max_over_ranks(f_ms + b_ms, dist, world)
    line = {
        "metric": "cell-updates/s (fwd+bwd, differentiable unroll 1024^2, C=3, K=9, T=64, "
                  "checkpoints every 8)",
        "value": world * n * n * T / (tot / 1e3), "unit": UNIT, "n_gpus": world,
        "steps": iters, "warmup": max(args.warmup, 3), "ms_per_step": tot,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
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
        "loss": float(loss.detach()),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_search(args):
    """Batched gradient search: 32 candidates at 1024^2, C=3, K=9, T=128,
    checkpoints every 16, MSE to the seed shifted by (+16, +8) px, Adam on
    the seed, mu, sigma, weights and ring weights; every iteration of all
    candidates is one CUDA graph (Adam included).  fwd+bwd cell-updates/s =
    candidates * n^2 * T / iteration time, against the plain per-creature
    loop (torch autograd over the same kernels + torch.optim.Adam, one
    candidate at a time)."""
    import torch
    world, rank, local, dist = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    from cella_nova_gb300 import _abi
    from cella_nova_gb300.autograd import DiffusionLeniaGPU
    from cella_nova_gb300.creature import make_creature
    from cella_nova_gb300.search import AdamConfig, GradientSearch
    n, C, T, every, ncand = 1024, 3, 128, 16, args.candidates
    t0 = time.perf_counter()
    dev = torch.device("cuda", local)
    crs = [make_creature(n, C, seed=5000 + 100 * rank + i, temp=1.0, device=dev)
           for i in range(ncand)]
    tgs = [np.roll(cr.seed, (8, 16), axis=(1, 2)) for cr in crs]
    gen_s = time.perf_counter() - t0
    adam = AdamConfig(lr_seed=1e-3, lr_params=1e-3, lr_rings=1e-2)
    sampler = ClockSampler(local)
    sampler.start()
    gs = GradientSearch(crs, tgs, T=T, every=every, adam=adam, n_streams=4)
    warm = max(args.warmup, 3)
    gs.run(1)                         # the first iteration eagerly (allocates scratch)
    loss_first = float(np.mean(gs.losses()))
    gs.run(warm - 1)                  # capture, then replays
    torch.cuda.synchronize()
    barrier(dist, world)
    iters = max(1, args.steps)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_wall0 = time.perf_counter()
    e0.record()
    gs.run(iters)
    e1.record()
    e1.synchronize()
    t_wall1 = time.perf_counter()
    barrier(dist, world)
    ms = max_over_ranks(e0.elapsed_time(e1), dist, world) / iters
    clocks = sampler.summary(t_wall0, t_wall1)
    losses = gs.losses()
    # mass of x_T against the seed it started from, FP64 on the GPU
    lib = _abi.load()
    # (x_T of the last iteration against the x_0 it was unrolled from, the
    # first checkpoint)
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

    # plain per-creature loop: torch autograd over the same adjoint kernels
    # and torch.optim.Adam, one candidate at a time (no graphs)
    plain_cands = min(ncand, 4)
    plain_ms = 0.0
    tgt = [torch.tensor(tg, dtype=torch.float32, device=dev) for tg in tgs[:plain_cands]]
    models = [DiffusionLeniaGPU(cr) for cr in crs[:plain_cands]]
    opts = [torch.optim.Adam([{"params": [m.seed], "lr": adam.lr_seed},
                              {"params": [m.mu, m.sigma, m.weights], "lr": adam.lr_params},
                              {"params": list(m.ring_weights), "lr": adam.lr_rings}])
            for m in models]

    def plain_iteration(i):
        m, opt = models[i], opts[i]
        opt.zero_grad(set_to_none=True)
        loss = torch.mean((m(T, every) - tgt[i]) ** 2)
        loss.backward()
        opt.step()

    for i in range(plain_cands):
        plain_iteration(i)
    torch.cuda.synchronize()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record()
    for i in range(plain_cands):
        plain_iteration(i)
    p1.record()
    p1.synchronize()
    plain_ms = p0.elapsed_time(p1) / plain_cands * ncand    # per iteration of all candidates
    del models, opts
    sampler.stop()

    cells = ncand * n * n * T
    value = world * cells / (ms / 1e3)
    line = {
        "metric": "cell-updates/s (batched gradient search fwd+bwd: 32 x 1024^2, C=3, K=9, "
                  "T=128, checkpoints every 16, in-graph Adam)",
        "value": value, "unit": UNIT, "n_gpus": world, "steps": iters, "warmup": warm,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{ncand} candidates 1024^2, 3 channels, 9 kernels (all pairs), "
                               "ring kernels built on the GPU each iteration, T=128, checkpoint "
                               "every 16, loss MSE vs seed shifted (+16,+8) px, Adam on seed, "
                               "mu, sigma, weights, ring weights; one CUDA graph per iteration "
                               "over 4 streams",
                   "step_unit": "one iteration (forward, backward, Adam) of every candidate",
                   "candidates": ncand},
        "plain_loop": {"value": world * cells / (plain_ms / 1e3), "unit": UNIT,
                       "ms_per_step": plain_ms,
                       "how": f"torch autograd + torch.optim.Adam per candidate, "
                              f"{plain_cands} candidates timed and scaled to {ncand}"},
        "batched_over_plain": plain_ms / ms,
        "loss_mean": float(np.mean(losses)),
        "loss_mean_first_iteration": loss_first,
        "iterations_total": warm + iters,
        "mass_drift_max": drift,
        # per candidate and iteration: builder 4, parameter fold 1, forward 4
        # per step, MSE 2, segment recompute 4 per step (3 for a segment's
        # last), backward 5 per step, kernel gradient 2, ring gradient 2, Adam
        # 3; plus the step counter once per iteration
        "gpu_launches": iters * (ncand * (13 * T - (T + every - 1) // every + 14) + 1),
        "clocks": clocks,
        "setup_s": {"generate": gen_s},
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"], line["grad_check"] = search_cpu_check(args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def search_cpu_check(args):
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
