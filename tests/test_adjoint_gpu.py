"""The hand-written adjoint kernels against FP64 autograd (oracle/autograd_ref.py,
itself pinned to the reference model's autograd and to finite differences)."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from cella_nova_gb300 import GpuMaceLenia  # noqa: E402
from cella_nova_gb300.autograd import DiffusionLeniaGPU, LeniaWorld  # noqa: E402
from cella_nova_gb300.creature import make_creature, ring_kernel  # noqa: E402
from oracle import autograd_ref as AR  # noqa: E402

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def spatial_kernels(cr):
    return np.stack([ring_kernel(cr.n, R, b) for R, b in zip(cr.ring_radius, cr.ring_weights)])


def test_single_step_vjp_matches_fp64():
    cr = make_creature(64, 3, seed=41, radius=(4, 12), seed_box=32, temp=1.3)
    dev = torch.device("cuda")
    h64 = spatial_kernels(cr)
    rng = np.random.default_rng(1)
    x = torch.tensor(cr.seed, dtype=torch.float32, device=dev)
    ybar = torch.tensor(rng.standard_normal(cr.seed.shape), dtype=torch.float32, device=dev)
    w = LeniaWorld(cr.n, cr.C, cr.c0, cr.c1, cr.temp)
    w.load(cr.mu, cr.sigma, cr.weights, torch.tensor(h64, dtype=torch.float32, device=dev))
    xbar = torch.empty_like(x)
    pgrad = torch.zeros(3 * cr.K, dtype=torch.float64, device=dev)
    kgrad = torch.zeros((cr.K, cr.n // 2, cr.n, 2), dtype=torch.float32, device=dev)
    lib = w.lib
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    assert lib.cg_step_backward(w.h, P(x), P(ybar), P(xbar), P(pgrad), P(kgrad)) == 0
    hbar = torch.empty((cr.K, cr.n, cr.n), dtype=torch.float32, device=dev)
    assert lib.cg_kernel_grad_spatial(w.h, P(kgrad), P(hbar)) == 0
    torch.cuda.synchronize()
    # FP64 reference: L = <ybar, step(x)>
    xt = torch.tensor(x.cpu().numpy().astype(np.float64), requires_grad=True)
    mu = torch.tensor(cr.mu.astype(np.float64), requires_grad=True)
    sg = torch.tensor(cr.sigma.astype(np.float64), requires_grad=True)
    ww = torch.tensor(cr.weights.astype(np.float64), requires_grad=True)
    ht = torch.tensor(h64, requires_grad=True)
    ks = torch.fft.fft2(ht.to(torch.complex128))
    out = AR.step(xt, ks, cr.c0, cr.c1, mu, sg, ww, cr.temp)
    L = torch.sum(out * torch.tensor(ybar.cpu().numpy().astype(np.float64)))
    gx, gmu, gsg, gw, gh = torch.autograd.grad(L, [xt, mu, sg, ww, ht])
    K = cr.K
    pg = pgrad.cpu().numpy()
    errs = {"x": rel(xbar.cpu(), gx), "mu": rel(pg[:K], gmu), "sigma": rel(pg[K:2 * K], gsg),
            "w": rel(pg[2 * K:], gw), "h": rel(hbar.cpu(), gh)}
    assert max(errs.values()) < 1e-4, errs
    w.close()


@pytest.mark.parametrize("n,C,T,every", [(64, 3, 6, 4), (128, 2, 9, 4), (128, 3, 64, 8)])
def test_unroll_gradients_match_fp64(n, C, T, every):
    cr = make_creature(n, C, seed=50 + n, radius=(n / 16, n / 6), seed_box=n // 2, temp=1.0)
    target = AR.shifted_target(cr.seed)
    ref = AR.gradients(cr, T, target)
    m = DiffusionLeniaGPU(cr)
    xT = m(T, every)
    loss = torch.mean((xT - torch.tensor(target, dtype=torch.float32, device="cuda")) ** 2)
    loss.backward()
    errs = {"loss": abs(float(loss.detach()) - ref["loss"]) / ref["loss"],
            "seed": rel(m.seed.grad.cpu(), ref["seed"]), "mu": rel(m.mu.grad.cpu(), ref["mu"]),
            "sigma": rel(m.sigma.grad.cpu(), ref["sigma"]),
            "weights": rel(m.weights.grad.cpu(), ref["weights"]),
            # jointly: a one-ring kernel is invariant to its weight (gradient 0)
            "ring": rel(np.concatenate([b.grad.cpu().numpy() for b in m.ring_weights]),
                        np.concatenate(ref["ring_weights"]))}
    print(errs)
    assert max(errs.values()) < 2e-3, errs


def test_unroll_forward_equals_graph_steps():
    """The differentiable unroll (kernels built on the GPU from the ring
    weights, parameters folded on the device) steps exactly like the graph
    path with the same kernels."""
    from cella_nova_gb300.orchestrator import creature_ring_specs
    cr = make_creature(128, 3, seed=60, radius=(8, 20), seed_box=64)
    m = DiffusionLeniaGPU(cr, autotune=False)   # the graph path below is untuned too
    with torch.no_grad():
        xT = m(7, 3)
    specs, w = creature_ring_specs(cr)
    wd = torch.tensor(w, device="cuda")
    torch.cuda.synchronize()
    with GpuMaceLenia.from_creature(cr) as sim:
        sim.build_ring_kernels(specs, wd.data_ptr())
        sim.run_steps(7)
        ref = sim.state()
    np.testing.assert_array_equal(xT.cpu().numpy(), ref)


def test_unroll_with_spatial_kernels_matches_fp64():
    """The kernel-agnostic path: spatial kernels h as a tensor (here the
    ring kernels; the library takes their spectra with its own FFTs),
    gradients against FP64 autograd."""
    from cella_nova_gb300.autograd import unroll
    n, C, T, every = 64, 2, 6, 4
    cr = make_creature(n, C, seed=77, radius=(4, 12), seed_box=32)
    target = AR.shifted_target(cr.seed)
    h64 = spatial_kernels(cr)
    ref = AR.gradients(cr, T, target, kspec=np.fft.fft2(h64))
    dev = torch.device("cuda")
    f32 = dict(dtype=torch.float32, device=dev)
    seed = torch.tensor(cr.seed, **f32, requires_grad=True)
    mu = torch.tensor(cr.mu, **f32, requires_grad=True)
    sg = torch.tensor(cr.sigma, **f32, requires_grad=True)
    ww = torch.tensor(cr.weights, **f32, requires_grad=True)
    h = torch.tensor(h64, device=dev, requires_grad=True)
    w = LeniaWorld(cr.n, cr.C, cr.c0, cr.c1, cr.temp)
    xT = unroll(w, seed, mu, sg, ww, h, T, every)
    loss = torch.mean((xT - torch.tensor(target, **f32)) ** 2)
    loss.backward()
    errs = {"seed": rel(seed.grad.cpu(), ref["seed"]), "mu": rel(mu.grad.cpu(), ref["mu"]),
            "sigma": rel(sg.grad.cpu(), ref["sigma"]), "weights": rel(ww.grad.cpu(), ref["weights"])}
    assert h.grad is not None and h.grad.shape == h.shape
    assert max(errs.values()) < 2e-3, errs
    w.close()
