"""Generate tests/golden/*.npz from the reference's own PyTorch model.

Run in a container where the reference checkout is available (it is not on
the GPU host): ``python tests/golden/make_golden.py /path/to/cella-nova``.

Each fixture runs train/diff_lenia_org.py's ``DiffusionLenia.step`` (with
``MCLenia.get_fftconv`` / ``growth`` from train/lenia_org.py:93-136) on a
seeded synthetic creature, the same way train/save_frames_png.py:185-199
drives it: parameters through the ``params`` dict, the kernel spectra written
over ``fft_kernel``.  Kernel k of the orchestrator API (input c0[k], output
c1[k]) sits at ``fft_kernel[0, c0[k], c1[k]]`` — dim 1 is the channel that is
transformed and summed over (lenia_org.py:131-134, diff_lenia_org.py:50).

Two runs per trajectory fixture: float64 (the pin for the FP64 oracle) and
float32 (the reference's own precision).  The grad_*.npz fixtures hold
gradients of MSE(x_T, seed shifted by (+16, +8) px) from the model's own
autograd in float64.  gauss_rings_*.npz hold kernel spectra from the
reference's kernel generator (train/generate_kernel_json.py:106-146), the
pin of the on-GPU kernel builder's Gaussian-ring family.
``pyperlin`` (used only for random initial
states, lenia_org.py:63-66) is replaced by an empty stub module because the
state is always given.
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from cella_nova_gb300.creature import make_creature  # noqa: E402


def load_reference(ref_root):
    stub = types.ModuleType("pyperlin")
    stub.FractalPerlin2D = object
    sys.modules.setdefault("pyperlin", stub)
    sys.path.insert(0, os.path.join(ref_root, "train"))
    import torch  # noqa: F401
    from diff_lenia_org import DiffusionLenia
    return DiffusionLenia


def run_reference(DL, cr, steps, dtype):
    import torch
    C, n = cr.C, cr.n
    cdt = torch.complex128 if dtype == torch.float64 else torch.complex64
    mu = np.zeros((1, C, C))
    sg = np.ones((1, C, C))
    w = np.zeros((1, C, C))
    kf = torch.zeros((1, C, C, n, n), dtype=cdt)
    for k in range(cr.K):
        i, o = int(cr.c0[k]), int(cr.c1[k])
        mu[0, i, o] = cr.mu[k]
        sg[0, i, o] = cr.sigma[k]
        w[0, i, o] = cr.weights[k]
        kf[0, i, o] = torch.from_numpy(cr.kspec[k].astype(np.complex128)).to(cdt)
    rings = 3
    params = {
        "k_size": 5,
        "mu": torch.from_numpy(mu).to(dtype),
        "sigma": torch.from_numpy(sg).to(dtype),
        "beta": torch.zeros((1, C, C, rings), dtype=dtype),
        "mu_k": torch.zeros((1, C, C, rings), dtype=dtype),
        "sigma_k": torch.ones((1, C, C, rings), dtype=dtype),
        "weights": torch.from_numpy(w).to(dtype),
    }
    state0 = torch.from_numpy(cr.seed[None]).to(dtype)
    m = DL(size=(1, n, n), dt=0.2, num_channels=C, params=params,
           state_init=state0, device="cpu")
    m.fft_kernel = kf
    m.temp = cr.temp
    wn = m.weights[0].detach().double().numpy()
    w_used = np.array([wn[int(cr.c0[k]), int(cr.c1[k])] for k in range(cr.K)])
    aff1 = m.compute_affinity()[0].detach().double().numpy()
    states = []
    for _ in range(steps):
        m.step()
        states.append(m.state[0].detach().double().numpy().copy())
    return np.stack(states), aff1, w_used


def reference_gradients(DL, cr, T, target):
    """Gradients of MSE(x_T, target) through the reference model's own
    autograd, w.r.t. the seed, mu, sigma and the (normalised) weights, which
    are swapped for leaf tensors after construction (all float64)."""
    import torch
    C, n = cr.C, cr.n
    dt = torch.float64
    mu = np.zeros((1, C, C))
    sg = np.ones((1, C, C))
    w = np.zeros((1, C, C))
    kf = torch.zeros((1, C, C, n, n), dtype=torch.complex128)
    for k in range(cr.K):
        i, o = int(cr.c0[k]), int(cr.c1[k])
        mu[0, i, o] = cr.mu[k]
        sg[0, i, o] = cr.sigma[k]
        w[0, i, o] = cr.weights[k]
        kf[0, i, o] = torch.from_numpy(cr.kspec[k].astype(np.complex128))
    params = {"k_size": 5, "mu": torch.from_numpy(mu), "sigma": torch.from_numpy(sg),
              "beta": torch.zeros((1, C, C, 3), dtype=dt), "mu_k": torch.zeros((1, C, C, 3), dtype=dt),
              "sigma_k": torch.ones((1, C, C, 3), dtype=dt), "weights": torch.from_numpy(w)}
    m = DL(size=(1, n, n), dt=0.2, num_channels=C, params=params,
           state_init=torch.from_numpy(cr.seed[None]).to(dt), device="cpu")
    seed_l = torch.from_numpy(cr.seed[None]).to(dt).requires_grad_(True)
    mu_l = torch.from_numpy(mu).requires_grad_(True)
    sg_l = torch.from_numpy(sg).requires_grad_(True)
    w_l = torch.from_numpy(w).requires_grad_(True)
    m.state, m.mu, m.sigma, m.weights = seed_l, mu_l, sg_l, w_l
    m.fft_kernel = kf
    m.temp = cr.temp
    for _ in range(T):
        m.step()
    loss = torch.mean((m.state[0] - torch.from_numpy(target)) ** 2)
    g = torch.autograd.grad(loss, [seed_l, mu_l, sg_l, w_l])
    pick = lambda a: np.array([a[0, int(cr.c0[k]), int(cr.c1[k])] for k in range(cr.K)])
    return (float(loss), g[0][0].numpy(), pick(g[1].numpy()), pick(g[2].numpy()),
            pick(g[3].numpy()))


GRAD_CASES = [
    # name, n, C, T, temp, radius, rng seed
    ("grad_c3k9_n32", 32, 3, 4, 1.0, (3.0, 7.0), 21),
    ("grad_c2k4_n64", 64, 2, 3, 1.4, (4.0, 12.0), 22),
]


CASES = [
    # name, n, C, steps, temp, radius, rng seed
    ("c3k9_n32", 32, 3, 4, 1.0, (3.0, 7.0), 11),
    ("c1k1_n16", 16, 1, 4, 0.7, (2.0, 5.0), 12),
    ("c2k4_n32", 32, 2, 4, 1.6, (3.0, 8.0), 13),
    ("c4k16_n64", 64, 4, 2, 1.0, (4.0, 12.0), 14),
]


# The ring radii and widths of ml-rs/example.rs:342-350 (global_r 10).
GAUSS_RADII = [0.25, 0.3167, 0.3833, 0.45, 0.5167, 0.5833, 0.65, 0.7167, 0.85]
GAUSS_WIDTHS = [0.03, 0.0411, 0.0522, 0.0633, 0.0744, 0.0856, 0.0967, 0.1078, 0.13]
GAUSS_CASES = [("gauss_rings_n64", 64, 10.0), ("gauss_rings_n128", 128, 25.0)]


def make_gauss_rings(ref_root):
    sys.path.insert(0, os.path.join(ref_root, "train"))
    from generate_kernel_json import generate_kernels_fft
    for name, n, global_r in GAUSS_CASES:
        ks = generate_kernels_fft(n, len(GAUSS_RADII), global_r, GAUSS_RADII, GAUSS_WIDTHS)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, n=n, global_r=global_r, radii=np.array(GAUSS_RADII),
                            widths=np.array(GAUSS_WIDTHS), kspec=np.stack(ks))
        print(f"wrote {path}")


def main(ref_root, only=None):
    if only in (None, "gauss"):
        make_gauss_rings(ref_root)
    if only == "gauss":
        return
    import torch
    DL = load_reference(ref_root)
    for name, n, C, steps, temp, radius, seed in CASES:
        cr = make_creature(n, C, seed=seed, radius=radius, temp=temp,
                           seed_box=n // 2)
        s64, a64, w64 = run_reference(DL, cr, steps, torch.float64)
        s32, a32, w32 = run_reference(DL, cr, steps, torch.float32)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(
            path, n=n, C=C, K=cr.K, temp=temp, seed=cr.seed, kspec=cr.kspec,
            c0=cr.c0, c1=cr.c1, mu=cr.mu, sigma=cr.sigma,
            weights_in=cr.weights, weights=w64, weights_f32=w32.astype(np.float32),
            states_f64=s64, aff1_f64=a64, states_f32=s32.astype(np.float32),
            aff1_f32=a32.astype(np.float32))
        print(f"wrote {path}: steps={steps}, mass0={cr.seed.sum(axis=(1, 2))}")
    for name, n, C, T, temp, radius, seed in GRAD_CASES:
        cr = make_creature(n, C, seed=seed, radius=radius, temp=temp, seed_box=n // 2)
        target = np.roll(cr.seed, (8, 16), axis=(1, 2))
        loss, gs, gm, gsg, gw = reference_gradients(DL, cr, T, target)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(
            path, n=n, C=C, K=cr.K, T=T, temp=temp, seed=cr.seed, kspec=cr.kspec,
            c0=cr.c0, c1=cr.c1, mu=cr.mu, sigma=cr.sigma, weights=cr.weights,
            ring_radius=cr.ring_radius,
            ring_w_flat=np.concatenate([np.asarray(b) for b in cr.ring_weights]),
            ring_w_len=np.array([len(b) for b in cr.ring_weights]),
            target=target, loss=loss, g_seed=gs, g_mu=gm, g_sigma=gsg, g_weights=gw)
        print(f"wrote {path}: loss={loss:.6e}")


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--only=")]
    only = next((a.split("=", 1)[1] for a in sys.argv[1:] if a.startswith("--only=")), None)
    if len(args) != 1:
        sys.exit("usage: make_golden.py /path/to/cella-nova [--only=NAME]")
    main(args[0], only)
