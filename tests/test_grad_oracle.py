"""Pin the FP64 gradient oracle (oracle/autograd_ref.py), CPU only.

(a) Against the reference's own PyTorch model: gradients of MSE(x_T, shifted
    seed) w.r.t. the seed, mu, sigma and weights from train/diff_lenia_org.py
    autograd (tests/golden/grad_*.npz).
(b) Against FP64 central finite differences (h = 1e-6) of the C oracle, for
    the ring weights and random directions of every other parameter.
"""
import glob
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from cella_nova_gb300.creature import Creature, ring_kernel  # noqa: E402
from oracle import autograd_ref as AR  # noqa: E402
from oracle import oracle as O  # noqa: E402

GRAD = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "grad_*.npz")))


def load_case(path):
    g = np.load(path)
    lens = g["ring_w_len"]
    flat = g["ring_w_flat"]
    rings, o = [], 0
    for L in lens:
        rings.append(flat[o:o + L].tolist())
        o += L
    cr = Creature(n=int(g["n"]), C=int(g["C"]), K=int(g["K"]), seed=g["seed"], kspec=g["kspec"],
                  c0=g["c0"], c1=g["c1"], mu=g["mu"], sigma=g["sigma"], weights=g["weights"],
                  temp=float(g["temp"]), ring_radius=g["ring_radius"], ring_weights=rings)
    return g, cr


@pytest.mark.parametrize("path", GRAD, ids=[os.path.basename(p) for p in GRAD])
def test_autograd_oracle_matches_reference_model_gradients(path):
    g, cr = load_case(path)
    out = AR.gradients(cr, int(g["T"]), g["target"], kspec=cr.kspec.astype(np.complex128))
    assert abs(out["loss"] - float(g["loss"])) <= 1e-12 * abs(float(g["loss"]))
    for name, ref in (("seed", g["g_seed"]), ("mu", g["g_mu"]), ("sigma", g["g_sigma"]),
                      ("weights", g["g_weights"])):
        got = out[name]
        err = np.abs(got - ref).max() / max(np.abs(ref).max(), 1e-300)
        assert err < 1e-9, (name, err)


def _loss_c(cr, T, target, mu, sigma, w, rings, seed):
    ks = np.stack([np.fft.fft2(ring_kernel(cr.n, R, b)) for R, b in zip(cr.ring_radius, rings)])
    x = seed
    for _ in range(T):
        x, _, _ = O.step_c(x, ks, cr.c0, cr.c1, mu, sigma, w, cr.temp)
    return np.mean((x - target) ** 2)


def test_autograd_oracle_matches_finite_differences():
    g, cr = load_case(GRAD[0])
    T = 3
    target = AR.shifted_target(cr.seed)
    out = AR.gradients(cr, T, target)
    rng = np.random.default_rng(0)
    h = 1e-6
    base = dict(mu=cr.mu.astype(np.float64), sigma=cr.sigma.astype(np.float64),
                w=cr.weights.astype(np.float64), rings=[list(b) for b in cr.ring_weights],
                seed=cr.seed.copy())

    def fd(mutate):
        p, m = {k: (v.copy() if isinstance(v, np.ndarray) else [list(b) for b in v])
                for k, v in base.items()}, None
        q = {k: (v.copy() if isinstance(v, np.ndarray) else [list(b) for b in v])
             for k, v in base.items()}
        mutate(p, +h)
        mutate(q, -h)
        lp = _loss_c(cr, T, target, p["mu"], p["sigma"], p["w"], p["rings"], p["seed"])
        lm = _loss_c(cr, T, target, q["mu"], q["sigma"], q["w"], q["rings"], q["seed"])
        return (lp - lm) / (2 * h)

    # seed along a random direction
    d = rng.standard_normal(cr.seed.shape)
    num = fd(lambda p, e: p.__setitem__("seed", p["seed"] + e * d))
    ana = float(np.sum(out["seed"] * d))
    assert abs(num - ana) <= 1e-6 * abs(ana) + 1e-12, (num, ana)
    for name, key in (("mu", "mu"), ("sigma", "sigma"), ("weights", "w")):
        d = rng.standard_normal(cr.K)
        num = fd(lambda p, e, key=key, d=d: p.__setitem__(key, p[key] + e * d))
        ana = float(np.dot(out[name], d))
        assert abs(num - ana) <= 1e-6 * abs(ana) + 1e-12, (name, num, ana)
    # every ring weight of the first two kernels
    for k in range(2):
        for l in range(len(cr.ring_weights[k])):
            def bump(p, e, k=k, l=l):
                p["rings"][k][l] += e
            num = fd(bump)
            ana = float(out["ring_weights"][k][l])
            assert abs(num - ana) <= 1e-5 * abs(ana) + 1e-11, (k, l, num, ana)
