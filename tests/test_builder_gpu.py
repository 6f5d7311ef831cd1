"""The on-GPU kernel builder (cg_build_ring_kernels) and the ring-weight
gradient (cg_ring_weight_grad), through the C ABI."""
import os

import numpy as np
import pytest

from cella_nova_gb300 import GpuMaceLenia
from cella_nova_gb300.creature import all_pairs, make_creature
from cella_nova_gb300.orchestrator import creature_ring_specs
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def conv_of(sim, K, n):
    return sim.download_conv_buffer().reshape(K, n, n)


@pytest.mark.parametrize("n,C,seed", [(64, 3, 1), (256, 2, 2), (1024, 3, 3)])
def test_shell_builder_matches_host_spectra(n, C, seed):
    import torch
    cr = make_creature(n, C, seed=seed, radius=(max(2.0, n / 16), max(4.0, n / 6)),
                       seed_box=n // 2)
    specs, w = creature_ring_specs(cr)
    wd = torch.tensor(w, device="cuda")
    torch.cuda.synchronize()
    with GpuMaceLenia.from_creature(cr) as a, GpuMaceLenia.from_creature(cr) as b:
        b.build_ring_kernels(specs, wd.data_ptr())
        ua, ub = conv_of(a, cr.K, n), conv_of(b, cr.K, n)
        scale = np.abs(ua).max()
        assert np.abs(ua - ub).max() <= 2e-6 * scale, np.abs(ua - ub).max() / scale
        # one step with the built kernels against the FP64 oracle (host spectra)
        x = b.state()
        b.iterate()
        ref, _, _ = (O.step_c if n <= 256 else O.step_np)(
            x.astype(np.float64), cr.kspec.astype(np.complex128), cr.c0, cr.c1,
            cr.mu.astype(np.float64), cr.sigma.astype(np.float64),
            cr.weights.astype(np.float64), cr.temp)
        assert np.abs(b.state() - ref).max() <= 1e-5


@pytest.mark.parametrize("name", ["gauss_rings_n64", "gauss_rings_n128"])
def test_gauss_builder_matches_reference_generator(name):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    n, gr = int(g["n"]), float(g["global_r"])
    K, C = len(g["radii"]), 3
    c0, c1 = all_pairs(C)
    cr = make_creature(n, C, seed=7, c0=c0, c1=c1, radius=(3, 6), seed_box=n // 2)
    specs = [(1, 1, gr * r, wd) for r, wd in zip(g["radii"], g["widths"])]
    with GpuMaceLenia.from_creature(cr) as a, GpuMaceLenia.from_creature(cr) as b:
        for k in range(K):
            a.set_kernel(g["kspec"][k], k)
        b.build_ring_kernels(specs)
        ua, ub = conv_of(a, K, n), conv_of(b, K, n)
        assert np.abs(ua - ub).max() <= 2e-6 * np.abs(ua).max()


def test_builder_all_ones_and_rebuild():
    """NULL ring weights mean all ones; building twice gives the same bits."""
    import torch
    cr = make_creature(128, 2, seed=9, radius=(6, 20), seed_box=64)
    specs, _ = creature_ring_specs(cr)
    ones = torch.ones((cr.K, 8), device="cuda")
    torch.cuda.synchronize()
    with GpuMaceLenia.from_creature(cr) as a, GpuMaceLenia.from_creature(cr) as b:
        a.build_ring_kernels(specs)
        b.build_ring_kernels(specs, ones.data_ptr())
        ua = conv_of(a, cr.K, 128)
        np.testing.assert_array_equal(ua, conv_of(b, cr.K, 128))
        a.build_ring_kernels(specs)
        np.testing.assert_array_equal(conv_of(a, cr.K, 128), ua)


def test_ring_weight_grad_matches_torch_autograd():
    import torch
    from cella_nova_gb300.autograd import RingKernelBuilder
    n = 64
    cr = make_creature(n, 2, seed=11, radius=(4, 14), seed_box=32)
    specs, w = creature_ring_specs(cr)
    rng = np.random.default_rng(0)
    hbar = rng.standard_normal((cr.K, n, n)).astype(np.float32)
    wd = torch.tensor(w, device="cuda")
    hb = torch.tensor(hbar, device="cuda")
    grad = torch.zeros((cr.K, 8), device="cuda")
    torch.cuda.synchronize()
    with GpuMaceLenia.from_creature(cr) as sim:
        sim.build_ring_kernels(specs, wd.data_ptr())
        sim.ring_weight_grad(hb.data_ptr(), grad.data_ptr(), wd.data_ptr())
        sim.synchronize()
    got = grad.cpu().numpy()
    builder = RingKernelBuilder(n, cr.ring_radius, [len(b) for b in cr.ring_weights])
    bs = [torch.tensor(np.asarray(b, np.float64), requires_grad=True) for b in cr.ring_weights]
    loss = (builder(bs) * torch.from_numpy(hbar.astype(np.float64))).sum()
    loss.backward()
    for k, b in enumerate(bs):
        ref = b.grad.numpy()
        B = len(ref)
        np.testing.assert_allclose(got[k, :B], ref, rtol=1e-4, atol=1e-4 * np.abs(ref).max())
        assert (got[k, B:] == 0).all()


@pytest.mark.parametrize("n,C,seed,var", [(64, 3, 11, None), (512, 2, 12, None),
                                          (512, 2, 13, [2, 3, 3, 3]), (512, 3, 14, [3, 4, 4, 1])])
def test_spatial_kernels_on_the_gpu_match_oracle(n, C, seed, var):
    """cg_set_kernels_spatial_device: the spectra of spatial kernels (the
    creature's rings, with no normaliser applied) taken by the library's own
    FFTs step within the bar of the FP64 oracle run on their FP64 fft2, and
    the convolutions agree with those of cg_set_kernel's host spectra.  The
    transform runs the handle's forward row pass in whatever variant it is
    set to (here also the streamed and the paired-row forms)."""
    import torch
    from cella_nova_gb300.creature import ring_kernel
    cr = make_creature(n, C, seed=seed, radius=(max(2.0, n / 16), max(4.0, n / 6)),
                       seed_box=n // 2)
    h64 = np.stack([ring_kernel(n, R, b) for R, b in zip(cr.ring_radius, cr.ring_weights)])
    hd = torch.tensor(h64, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    with GpuMaceLenia.from_creature(cr) as a, GpuMaceLenia.from_creature(cr) as b:
        if var is not None:
            b.set_variants(var)
        b.set_kernels_spatial_device(hd.data_ptr())
        ua, ub = conv_of(a, cr.K, n), conv_of(b, cr.K, n)
        assert np.abs(ua - ub).max() <= 2e-6 * np.abs(ua).max()
        x = b.state()
        b.iterate()
        ref, _, _ = (O.step_c if n <= 256 else O.step_np)(
            x.astype(np.float64), np.fft.fft2(h64), cr.c0, cr.c1, cr.mu.astype(np.float64),
            cr.sigma.astype(np.float64), cr.weights.astype(np.float64), cr.temp)
        assert np.abs(b.state() - ref).max() <= 1e-5
