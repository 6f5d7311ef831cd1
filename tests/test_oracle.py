"""Pin the CPU oracle against the reference's own model (CPU only).

tests/golden/*.npz were produced by train/diff_lenia_org.py's
DiffusionLenia (tests/golden/make_golden.py).  The C restatement of
ml-rs/example.rs (FP64) and its numpy twin must reproduce the reference's
float64 run to round-off; the FP32 build must stay within the reference's own
float32 spread.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = sorted(p for p in glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))
                if not os.path.basename(p).startswith(("grad_", "gauss_")))


def _args(g):
    return (g["c0"], g["c1"], g["mu"].astype(np.float64), g["sigma"].astype(np.float64),
            g["weights"], float(g["temp"]))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_c_oracle_f64_matches_reference_model(path):
    g = np.load(path)
    st = g["seed"].copy()
    ks = g["kspec"].astype(np.complex128)
    for t in range(g["states_f64"].shape[0]):
        st, _, aff = O.step_c(st, ks, *_args(g), want_aff=True)
        if t == 0:
            np.testing.assert_allclose(aff, g["aff1_f64"], rtol=0, atol=1e-12)
        np.testing.assert_allclose(st, g["states_f64"][t], rtol=0, atol=1e-12)


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_numpy_twin_matches_reference_model(path):
    g = np.load(path)
    st = g["seed"].copy()
    ks = g["kspec"].astype(np.complex128)
    for t in range(g["states_f64"].shape[0]):
        st, _, _ = O.step_np(st, ks, *_args(g))
        np.testing.assert_allclose(st, g["states_f64"][t], rtol=0, atol=1e-12)


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_c_oracle_f32_within_reference_f32_spread(path):
    g = np.load(path)
    st = g["seed"].astype(np.float32)
    ks = g["kspec"].astype(np.complex128)
    for t in range(g["states_f64"].shape[0]):
        st, _, _ = O.step_c(st, ks, *_args(g), dtype=np.float32)
        # the reference's float32 run differs from its float64 run by ~2e-6
        assert np.abs(st - g["states_f64"][t]).max() < 1e-5
        assert np.abs(g["states_f32"][t] - g["states_f64"][t]).max() < 1e-5


def test_faithful_and_shared_spectrum_orders_agree():
    g = np.load(GOLDEN[0])
    ks = g["kspec"].astype(np.complex128)
    a, _, _ = O.step_c(g["seed"], ks, *_args(g), faithful=True)
    b, _, _ = O.step_c(g["seed"], ks, *_args(g), faithful=False, nthreads=2)
    np.testing.assert_array_equal(a, b)


def test_oracle_conserves_mass():
    g = np.load(GOLDEN[0])
    ks = g["kspec"].astype(np.complex128)
    st = g["seed"].copy()
    m0 = O.mass_c(st)
    for _ in range(10):
        st, _, _ = O.step_c(st, ks, *_args(g))
    np.testing.assert_allclose(O.mass_c(st), m0, rtol=1e-13)


def test_oracle_u_is_convolution():
    """u_k is the circular convolution of the input channel with kernel k."""
    rng = np.random.default_rng(3)
    n = 16
    x = rng.random((1, n, n))
    h = rng.random((n, n))
    ks = np.fft.fft2(h)[None]
    _, u, _ = O.step_c(x, ks, [0], [0], [0.1], [0.05], [1.0], 1.0, want_u=True)
    ref = np.zeros((n, n))
    for dy in range(n):
        for dx in range(n):
            ref += h[dy, dx] * np.roll(x[0], (dy, dx), axis=(0, 1))
    np.testing.assert_allclose(u[0], ref, atol=1e-12)


def test_loaders_swap_and_resample(tmp_path):
    from cella_nova_gb300.creature import make_creature, write_creature
    cr = make_creature(32, 2, seed=5, radius=(3, 6), seed_box=16)
    js, kb = write_creature(str(tmp_path), "t", cr)
    cfg = O.load_config_np(js)
    np.testing.assert_array_equal(cfg["c0"], cr.c0)
    np.testing.assert_array_equal(cfg["c1"], cr.c1)
    np.testing.assert_array_equal(cfg["seed"], cr.seed)
    k64 = O.load_kernels_np(kb, cr.K, 64)
    # zero-padding the centred spectrum = upsampling the kernel by 2 (sum x4)
    for k in range(cr.K):
        assert abs(k64[k][0, 0] - cr.kspec[k][0, 0]) < 1e-6
        np.testing.assert_allclose(np.fft.fftshift(k64[k])[16:48, 16:48],
                                   np.fft.fftshift(cr.kspec[k]), atol=0)


@pytest.mark.parametrize("name", ["gauss_rings_n64", "gauss_rings_n128"])
def test_gauss_ring_generator_restatement(name):
    """The kernel generator's Gaussian rings (generate_kernel_json.py:106-146)
    against the spectra the reference's own generator wrote."""
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", f"{name}.npz"))
    ks = O.gauss_ring_kernels_np(int(g["n"]), float(g["global_r"]), g["radii"], g["widths"])
    # the reference builds float32 values and stores complex64
    assert np.abs(ks - g["kspec"]).max() < 5e-7

