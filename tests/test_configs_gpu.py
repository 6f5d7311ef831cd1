"""The benchmark configurations' own checks, at their stated sizes.

* Plain DiffusionLenia at 1024^2, C=3, K=9, 200 steps, compared step by step
  with the FP64 oracle (ml-rs/example.rs:164-303, restated in oracle/): every
  step is teacher-forced (the oracle starts from the GPU's state), the
  per-step max-abs error stays within 1e-5 and the FP64 mass of the
  free-running GPU trajectory within 1e-6 relative.
* The reference's acceptance test (scripts/integration.sh:8-46,
  train/compare_pngs.py:72-78) at the sizes it runs, 1024^2 and 2048^2:
  50 free-running steps, every frame's 8-bit grey image within one grey
  level of the FP64 oracle's.
* The differentiable unroll's gradients on the 128^2 instance (C=3, K=9,
  T=64, checkpoints every 8) against FP64 central finite differences
  (h = 1e-6) of the C oracle: random directions of the seed, mu, sigma and
  the growth weights, and every ring weight of two kernels.
"""
import os

import numpy as np
import pytest

from cella_nova_gb300 import GpuMaceLenia
from cella_nova_gb300.creature import make_creature, ring_kernel
from oracle import oracle as O

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-5
THREADS = os.cpu_count() or 1


def oracle_args(cr):
    return (cr.kspec.astype(np.complex128), cr.c0, cr.c1, cr.mu.astype(np.float64),
            cr.sigma.astype(np.float64), cr.weights.astype(np.float64), cr.temp)


def test_plain_1024_two_hundred_steps_step_by_step():
    """200 steps at 1024^2 (ring radii U[12,30] px, seed on the central
    256^2 square, c0/c1 over every pair), each against the FP64 oracle from
    the same state."""
    cr = make_creature(1024, 3, seed=1024, temp=1.0)
    a = oracle_args(cr)
    errs = []
    with GpuMaceLenia.from_creature(cr) as sim:
        m0 = sim.mass_f64()
        x = sim.state()
        for _ in range(200):
            sim.iterate()
            y = sim.state()
            ref, _, _ = O.step_c(x.astype(np.float64), *a, nthreads=THREADS)
            errs.append(float(np.abs(y - ref).max()))
            x = y
        m1 = sim.mass_f64()
    errs = np.asarray(errs)
    drift = float(np.abs(m1 / m0 - 1).max())
    print(f"1024^2 C=3 K=9, 200 steps: per-step max-abs error max {errs.max():.3e}, "
          f"median {np.median(errs):.3e}; mass drift {drift:.2e}")
    assert errs.max() <= STEP_TOL, (int(errs.argmax()), errs.max())
    assert drift < 1e-6, drift
    assert np.isfinite(x).all() and x.max() > 0


def grey_frame(x):
    """The frame the reference's integration test compares
    (train/save_frames_png.py:202-210): the channel sum, min-max normalised
    to 0..255 and truncated to 8 bits."""
    img = x.sum(axis=0).astype(np.float64)
    lo, hi = img.min(), img.max()
    if hi <= lo:
        return np.zeros(img.shape, np.uint8)
    return ((img - lo) / (hi - lo) * 255).astype(np.uint8)


@pytest.mark.parametrize("n", [1024, 2048])
def test_acceptance_fifty_steps_at_reference_sizes(n):
    """The sizes scripts/integration.sh runs: the benchmark creatures at
    1024^2 and 2048^2, 50 free-running steps each."""
    cr = make_creature(n, 3, seed=4096 + n, temp=1.0)
    a = oracle_args(cr)
    x64 = cr.seed.astype(np.float64)
    worst = 0
    with GpuMaceLenia.from_creature(cr) as sim:
        for _ in range(50):
            sim.iterate()
            x64, _, _ = O.step_c(x64, *a, nthreads=THREADS)
            d = np.abs(grey_frame(sim.state()).astype(int) - grey_frame(x64).astype(int)).max()
            worst = max(worst, int(d))
        drift = float(np.abs(sim.state() - x64).max())
    print(f"{n}^2: worst grey-level difference {worst}, state max-abs {drift:.2e} after 50 steps")
    assert worst <= 1, worst
    assert drift <= 1e-4, drift


def _fd_loss(cr, T, target, mu, sigma, w, rings, seed):
    ks = np.stack([np.fft.fft2(ring_kernel(cr.n, R, b)) for R, b in zip(cr.ring_radius, rings)])
    x = seed
    for _ in range(T):
        x, _, _ = O.step_c(x, ks, cr.c0, cr.c1, mu, sigma, w, cr.temp, nthreads=THREADS)
    return float(np.mean((x - target) ** 2))


def test_unroll_gradients_match_finite_differences_128():
    """GPU gradients (adjoint kernels, f32) of MSE(x_T, seed shifted by
    (+16, +8) px) at 128^2, C=3, K=9, T=64, checkpoints every 8, against
    FP64 central differences of the C oracle, h = 1e-6.  Each directional
    derivative must agree to 1e-4 of the scale sum_i |g_i d_i| (the size of
    the terms the derivative sums, so cancellation cannot hide an error)."""
    torch = pytest.importorskip("torch")
    from cella_nova_gb300.autograd import DiffusionLeniaGPU
    from oracle import autograd_ref as AR
    n, C, T, every, h = 128, 3, 64, 8, 1e-6
    cr = make_creature(n, C, seed=128, radius=(n / 16, n / 6), seed_box=n // 2, temp=1.0)
    target = AR.shifted_target(cr.seed)
    m = DiffusionLeniaGPU(cr)
    xT = m(T, every)
    loss = torch.mean((xT - torch.tensor(target, dtype=torch.float32, device="cuda")) ** 2)
    loss.backward()
    g = {"seed": m.seed.grad.double().cpu().numpy(), "mu": m.mu.grad.double().cpu().numpy(),
         "sigma": m.sigma.grad.double().cpu().numpy(),
         "weights": m.weights.grad.double().cpu().numpy(),
         "rings": [b.grad.double().cpu().numpy() for b in m.ring_weights]}
    base = {"mu": cr.mu.astype(np.float64), "sigma": cr.sigma.astype(np.float64),
            "weights": cr.weights.astype(np.float64), "seed": cr.seed.astype(np.float64)}

    def central(key, d=None, ring=None):
        vals = []
        for e in (+h, -h):
            p = {k: v.copy() for k, v in base.items()}
            rings = [list(b) for b in cr.ring_weights]
            if ring is None:
                p[key] = p[key] + e * d
            else:
                rings[ring[0]][ring[1]] += e
            vals.append(_fd_loss(cr, T, target, p["mu"], p["sigma"], p["weights"], rings,
                                 p["seed"]))
        return (vals[0] - vals[1]) / (2 * h)

    rng = np.random.default_rng(5)
    report = {}
    for key in ("seed", "mu", "sigma", "weights"):
        d = rng.standard_normal(base[key].shape)
        num = central(key, d)
        ana = float(np.sum(g[key] * d))
        scale = float(np.sum(np.abs(g[key] * d)))
        report[key] = (num, ana, abs(num - ana) / scale)
    # a one-ring kernel is invariant to its weight (the kernel is normalised),
    # so ring derivatives are measured against the largest of them
    ring_scale = max(float(np.abs(b).max()) for b in g["rings"][:2])
    for k in range(2):
        for l in range(len(cr.ring_weights[k])):
            num = central(None, ring=(k, l))
            ana = float(g["rings"][k][l])
            report[f"ring{k}.{l}"] = (num, ana,
                                      abs(num - ana) / max(abs(num), 1e-2 * ring_scale))
    print({k: f"fd {v[0]:.6e} gpu {v[1]:.6e} err {v[2]:.1e}" for k, v in report.items()})
    bad = {k: v for k, v in report.items() if not v[2] <= 1e-4}
    assert not bad, bad
