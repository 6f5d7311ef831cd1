"""The batched gradient search (cella_nova_gb300/search.py): its gradients
against FP64 autograd (oracle/autograd_ref.py), its Adam step against
torch.optim.Adam, and graph replays against eager iterations."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from cella_nova_gb300 import _abi  # noqa: E402
from cella_nova_gb300.creature import make_creature  # noqa: E402
from cella_nova_gb300.search import AdamConfig, GradientSearch  # noqa: E402
from oracle import autograd_ref as AR  # noqa: E402

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def candidates(n, C, count, seed0=60):
    crs = [make_creature(n, C, seed=seed0 + i, radius=(max(2.0, n / 16), max(4.0, n / 5)),
                         seed_box=n // 2, temp=1.0 + 0.25 * i) for i in range(count)]
    return crs, [AR.shifted_target(cr.seed) for cr in crs]


@pytest.mark.parametrize("n,C,T,every", [(64, 2, 8, 4), (128, 3, 6, 4)])
def test_search_gradients_match_fp64_autograd(n, C, T, every):
    crs, tgs = candidates(n, C, 2)
    with GradientSearch(crs, tgs, T=T, every=every, n_streams=2) as gs:
        gs.run_eager(1)    # gradients at the initial parameters
        for i, (cr, tg) in enumerate(zip(crs, tgs)):
            got = gs.gradients(i)
            ref = AR.gradients(cr, T, tg, ring=True)
            assert abs(got["loss"] / ref["loss"] - 1) < 1e-4
            errs = {k: rel(got[k], ref[k]) for k in ("seed", "mu", "sigma", "weights")}
            gr = np.concatenate([got["ring_weights"][k, :len(b)]
                                 for k, b in enumerate(ref["ring_weights"])])
            errs["ring"] = rel(gr, np.concatenate(ref["ring_weights"]))
            assert max(errs.values()) < 2e-3, errs


def test_adam_step_matches_torch_adam():
    lib = _abi.load()
    rng = np.random.default_rng(5)
    cfg = dict(lr=3e-3, betas=(0.9, 0.99), eps=1e-8)
    p0 = rng.standard_normal(1000).astype(np.float32)
    grads = [rng.standard_normal(1000) for _ in range(4)]
    ref = torch.tensor(p0, requires_grad=True)
    opt = torch.optim.Adam([ref], **cfg)
    for gf64 in (False, True):
        p = torch.tensor(p0, device="cuda")
        m, v = torch.zeros_like(p), torch.zeros_like(p)
        step = torch.zeros(1, dtype=torch.int32, device="cuda")
        for g in grads:
            gd = torch.tensor(g, dtype=torch.float64 if gf64 else torch.float32, device="cuda")
            ptr = ctypes.c_void_p(gd.data_ptr())
            torch.cuda.synchronize()
            _abi.check(lib.cg_adam_step(ctypes.c_void_p(p.data_ptr()), None if gf64 else ptr,
                                        ptr if gf64 else None, ctypes.c_void_p(m.data_ptr()),
                                        ctypes.c_void_p(v.data_ptr()), p.numel(),
                                        ctypes.c_float(cfg["lr"]), ctypes.c_float(0.9),
                                        ctypes.c_float(0.99), ctypes.c_float(1e-8),
                                        ctypes.c_void_p(step.data_ptr()), None))
            _abi.check(lib.cg_count_step(ctypes.c_void_p(step.data_ptr()), None))
        torch.cuda.synchronize()
        if not gf64:
            for g in grads:
                ref.grad = torch.tensor(g, dtype=torch.float32)
                opt.step()
        assert int(step.item()) == 4
        np.testing.assert_allclose(p.cpu().numpy(), ref.detach().numpy(), rtol=1e-5, atol=1e-6)


def test_mse_grad_and_loss():
    lib = _abi.load()
    rng = np.random.default_rng(6)
    x = rng.standard_normal(12345).astype(np.float32)
    t = rng.standard_normal(12345).astype(np.float32)
    xd, td = torch.tensor(x, device="cuda"), torch.tensor(t, device="cuda")
    g = torch.empty_like(xd)
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    scratch = torch.zeros(_abi.REDUCE_BLOCKS, dtype=torch.float64, device="cuda")
    P = lambda a: ctypes.c_void_p(a.data_ptr())
    torch.cuda.synchronize()
    _abi.check(lib.cg_mse_grad(P(xd), P(td), x.size, P(g), P(loss), P(scratch), None))
    torch.cuda.synchronize()
    d = (x - t).astype(np.float64)          # the difference is taken in f32
    assert abs(loss.item() - (d * d).mean()) <= 1e-12 * (d * d).mean()
    np.testing.assert_allclose(g.cpu().numpy(), 2 * (x - t) / x.size, rtol=1e-6)


def test_graph_replays_equal_eager_iterations_and_conserve_mass():
    crs, tgs = candidates(64, 3, 3)
    adam = AdamConfig(lr_seed=1e-2, lr_params=1e-3, lr_rings=1e-2)
    # untuned: both on the same variants, and no tuning time in the test
    with GradientSearch(crs, tgs, T=8, every=4, adam=adam, n_streams=2, autotune=False) as a, \
            GradientSearch(crs, tgs, T=8, every=4, adam=adam, n_streams=2, autotune=False) as b:
        a.run(5)          # one eager iteration, then four replays of the captured graph
        b.run_eager(5)
        assert a.graph is not None and b.graph is None
        for i in range(3):
            pa, pb = a.parameters(i), b.parameters(i)
            for k in pa:
                # growth-gradient sums use FP64 atomics: equal to round-off
                np.testing.assert_allclose(pa[k], pb[k], rtol=1e-5, atol=1e-6, err_msg=k)
            ga = a.gradients(i)
            # the unroll conserves each channel's mass
            m0 = ga["initial"].astype(np.float64).sum(axis=(1, 2))
            mT = ga["final"].astype(np.float64).sum(axis=(1, 2))
            assert np.abs(mT / m0 - 1).max() < 1e-6


def test_loss_decreases():
    crs, tgs = candidates(64, 2, 2, seed0=80)
    adam = AdamConfig(lr_seed=2e-2, lr_params=2e-3, lr_rings=2e-2)
    with GradientSearch(crs, tgs, T=8, every=4, adam=adam) as gs:
        gs.run(1)
        first = gs.losses()
        gs.run(30)
        last = gs.losses()
    assert (last < 0.8 * first).all(), (first, last)
