"""Parity of the CUDA step against the FP64 oracle, through the C ABI.

Every comparison is teacher-forced: the GPU and the oracle start each step
from the same state (the GPU's f32 state, widened to f64 for the oracle), so
the difference measures one step's error, which the bar puts at max-abs
1e-5 (the dynamics are chaotic, so whole trajectories are compared only
through size-independent properties such as mass).
"""
import os

import numpy as np
import pytest

from cella_nova_gb300 import GpuMaceLenia, setup_simulation
from cella_nova_gb300.creature import all_pairs, make_creature, write_creature
from oracle import oracle as O

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-5          # max-abs per step against FP64
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def oracle_step(state, cr, want_u=False, want_aff=False):
    fn = O.step_c if cr.n <= 256 else O.step_np
    return fn(state.astype(np.float64), cr.kspec.astype(np.complex128), cr.c0, cr.c1,
              cr.mu.astype(np.float64), cr.sigma.astype(np.float64),
              cr.weights.astype(np.float64), cr.temp, want_u=want_u, want_aff=want_aff)


def check_steps(cr, steps=3, tol=STEP_TOL):
    with GpuMaceLenia.from_creature(cr) as sim:
        errs = []
        for _ in range(steps):
            x = sim.state()
            sim.iterate()
            got = sim.state()
            ref, _, _ = oracle_step(x, cr)
            errs.append(np.abs(got - ref).max())
        assert max(errs) <= tol, errs
        return errs


@pytest.mark.parametrize("name", ["c1k1_n16", "c3k9_n32", "c2k4_n32", "c4k16_n64"])
def test_golden_trajectory_from_reference_model(name):
    """The GPU path against the reference's own PyTorch model (float64)."""
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    n, C = int(g["n"]), int(g["C"])
    with GpuMaceLenia((n, n), C, int(g["K"]), g["c0"], g["c1"], g["mu"], g["sigma"],
                      g["weights"].astype(np.float32), float(g["temp"])) as sim:
        for k in range(int(g["K"])):
            sim.set_kernel(g["kspec"][k], k)
        sim.upload_state(g["seed"])
        for t in range(g["states_f64"].shape[0]):
            sim.iterate()
            err = np.abs(sim.state() - g["states_f64"][t]).max()
            # a few steps of free-running f32 against f64: same spread as the
            # reference's own float32 run
            ref32 = np.abs(g["states_f32"][t] - g["states_f64"][t]).max()
            assert err <= max(4 * ref32, STEP_TOL), (t, err, ref32)


@pytest.mark.parametrize("n,C,seed,temp", [
    (16, 1, 1, 1.0), (32, 2, 2, 0.5), (64, 3, 3, 1.0), (64, 4, 4, 2.0),
    (128, 3, 5, 1.0), (256, 3, 6, 1.3), (256, 1, 7, 0.8),
])
def test_step_parity_all_pairs(n, C, seed, temp):
    cr = make_creature(n, C, seed=seed, temp=temp, radius=(max(2.0, n / 16), max(4.0, n / 6)),
                       seed_box=n // 2)
    check_steps(cr)


@pytest.mark.parametrize("c0,c1", [
    ([1, 0, 2, 1], [0, 1, 1, 2]),          # the reference's reverse slot copy mishandles this
    ([2, 2, 2], [0, 0, 0]),                 # one input feeds one output three times
    ([0], [2]),                             # channels 0 and 1 get no growth term
    ([0, 1, 2, 0, 1, 2, 0, 1, 2, 2, 1], [0, 0, 0, 1, 1, 1, 2, 2, 2, 0, 1]),   # K != C^2
])
def test_step_parity_irregular_maps(c0, c1):
    cr = make_creature(64, 3, seed=17, c0=c0, c1=c1, radius=(4, 12), seed_box=32)
    check_steps(cr)


def test_many_kernels_and_channels():
    C = 8
    c0 = np.repeat(np.arange(C), 5) % C
    c1 = (np.arange(5 * C) * 3) % C
    cr = make_creature(64, C, seed=21, c0=c0, c1=c1, radius=(3, 10), seed_box=32)
    check_steps(cr, steps=2)


def test_conv_buffer_and_affinity_match_oracle():
    cr = make_creature(128, 3, seed=8, radius=(8, 20), seed_box=64)
    with GpuMaceLenia.from_creature(cr) as sim:
        x = sim.state()
        conv = sim.download_conv_buffer().reshape(cr.K, 128, 128)
        aff = sim.download_affinity().reshape(cr.C, 128, 128)
        np.testing.assert_array_equal(sim.state(), x)      # debug reads do not step
    _, u, A = oracle_step(x, cr, want_u=True, want_aff=True)
    # download_conv_buffer is the unscaled IFFT (growth.rs:87 scales by 1/n^2)
    assert np.abs(conv / (128 * 128) - u).max() < 1e-6
    assert np.abs(aff - A).max() / np.abs(A).max() < 1e-5


@pytest.mark.parametrize("nsteps", [4, 9, 17])
def test_graph_steps_equal_timed_and_stream_steps(nsteps):
    """Per-channel pipelined graphs (8 steps and 1 step) against one launch
    per phase, step by step."""
    cr = make_creature(128, 3, seed=9, radius=(8, 20), seed_box=64)
    with GpuMaceLenia.from_creature(cr) as a, GpuMaceLenia.from_creature(cr) as b, \
            GpuMaceLenia.from_creature(cr) as c:
        a.run_steps(nsteps)
        for _ in range(nsteps):
            ms = b.timed_iterate()
            assert ms.shape == (4,) and ms[3] == 0.0 and (ms[:3] >= 0).all()
        import torch
        s = torch.cuda.Stream()
        for _ in range(nsteps):
            c.iterate_on(s.cuda_stream)
        s.synchronize()
        np.testing.assert_array_equal(a.state(), b.state())
        np.testing.assert_array_equal(a.state(), c.state())


def test_mass_f64_matches_host_sum_and_is_conserved():
    cr = make_creature(256, 3, seed=10, radius=(10, 30), seed_box=128)
    with GpuMaceLenia.from_creature(cr) as sim:
        m0 = sim.mass_f64()
        np.testing.assert_allclose(m0, sim.state().astype(np.float64).sum(axis=(1, 2)),
                                   rtol=1e-12)
        sim.run_steps(200)
        m1 = sim.mass_f64()
        assert np.abs(m1 / m0 - 1).max() < 1e-6


def test_reference_files_through_setup_simulation(tmp_path):
    cr = make_creature(64, 3, seed=11, radius=(4, 12), seed_box=32, temp=1.5)
    js, kb = write_creature(str(tmp_path), "crit", cr)
    sim = setup_simulation(js, kb)
    try:
        assert abs(sim.temp - 1.5) < 1e-7
        x = sim.state()
        np.testing.assert_array_equal(x, cr.seed.astype(np.float32))
        sim.iterate()
        ref, _, _ = oracle_step(x, cr)
        assert np.abs(sim.state() - ref).max() <= STEP_TOL
    finally:
        sim.close()


@pytest.mark.parametrize("n", [1024, 2048])
def test_full_size_step_parity(n):
    """The benchmark configurations (3 channels, 9 kernels) at full size."""
    cr = make_creature(n, 3, seed=100 + n, temp=1.0)
    check_steps(cr, steps=1)


def test_mass_drift_1000_steps_2048():
    cr = make_creature(2048, 3, seed=2048, temp=1.0)
    with GpuMaceLenia.from_creature(cr) as sim:
        m0 = sim.mass_f64()
        sim.run_steps(1000)
        m1 = sim.mass_f64()
        x = sim.state()
    assert np.isfinite(x).all()
    assert np.abs(m1 / m0 - 1).max() < 1e-6, m1 / m0 - 1


def test_kernel_reupload_and_zero_kernel():
    """set_kernel overwrites; an all-zero spectrum gives u = 0 everywhere."""
    cr = make_creature(64, 2, seed=12, radius=(4, 10), seed_box=32)
    with GpuMaceLenia.from_creature(cr) as sim:
        sim.set_kernel(np.zeros((64, 64), np.complex64), 0)
        conv = sim.download_conv_buffer().reshape(cr.K, 64, 64)
        assert np.abs(conv[0]).max() == 0.0
        sim.set_kernel(cr.kspec[0], 0)
        conv = sim.download_conv_buffer().reshape(cr.K, 64, 64)
        assert np.abs(conv[0]).max() > 0.0


@pytest.mark.parametrize("n", [16, 32, 64, 256, 1024, 2048])
def test_variants_agree_and_autotune(n):
    """Every CTA-shape variant (0-2, and diffusion's 3) computes the same
    bits; the autotuner keeps a variant of each phase that exists at this
    size and does not step the world."""
    cr = make_creature(n, 3, seed=70 + n, radius=(max(2.0, n / 16), max(4.0, n / 6)),
                       seed_box=n // 2)
    with GpuMaceLenia.from_creature(cr) as sim:
        assert sim.variants() == [0, 0, 0, 0]
        sim.run_steps(3)
        ref = sim.state()
    for p in range(4):
        for v in ((1, 2, 3) if p == 3 else (1, 2)):
            var = [0, 0, 0, 0]
            var[p] = v
            with GpuMaceLenia.from_creature(cr) as sim:
                sim.set_variants(var)
                sim.run_steps(3)
                np.testing.assert_array_equal(sim.state(), ref, err_msg=str(var))
    counts = [4 if p == 3 else (5 if n >= 512 else 3) for p in range(4)]
    with GpuMaceLenia.from_creature(cr) as sim:
        x0 = sim.state()
        chosen, ms = sim.autotune(reps=3)
        np.testing.assert_array_equal(sim.state(), x0)    # tuning does not step
        assert ms.shape == (4, 5)
        for p in range(4):
            assert 0 <= chosen[p] < counts[p]
            assert (ms[p, :counts[p]] > 0).all() and (ms[p, counts[p]:] == -1).all()
        assert sim.variants() == chosen
        sim.run_steps(3)
        if max(chosen[:3]) <= 2:
            np.testing.assert_array_equal(sim.state(), ref)
        else:   # an FFT-plan variant: the same step to rounding
            assert np.abs(sim.state() - ref).max() <= 3 * STEP_TOL


@pytest.mark.parametrize("n", [512, 1024, 2048])
def test_plan_variants_match_oracle(n):
    """The FFT-plan variants (3: paired rows, radix 16 / swapped column
    plans; 4: paired rows, radix 8 / swapped plans in another CTA shape),
    alone and together, step by step against the FP64 oracle."""
    cr = make_creature(n, 3, seed=90 + n, temp=1.0)
    a = (cr.kspec.astype(np.complex128), cr.c0, cr.c1, cr.mu.astype(np.float64),
         cr.sigma.astype(np.float64), cr.weights.astype(np.float64), cr.temp)
    combos = [[3, 0, 0, 0], [4, 0, 0, 0], [0, 3, 0, 0], [0, 4, 0, 0], [0, 0, 3, 0],
              [0, 0, 4, 0], [3, 3, 3, 1], [4, 4, 4, 1]]
    worst = {}
    for var in combos:
        with GpuMaceLenia.from_creature(cr) as sim:
            sim.set_variants(var)
            assert sim.variants() == var
            sim.run_steps(2)
            errs = []
            for _ in range(2):
                x = sim.state()
                sim.iterate()
                ref, _, _ = O.step_c(x.astype(np.float64), *a, nthreads=os.cpu_count() or 1)
                errs.append(float(np.abs(sim.state() - ref).max()))
            worst[str(var)] = max(errs)
            if n == 512 and var[2] >= 3:
                # the debug buffer of the paired inverse row pass
                x = sim.state()
                conv = sim.download_conv_buffer().reshape(cr.K, n, n)
                _, u, _ = oracle_step(x, cr, want_u=True)
                worst[f"{var} u"] = float(np.abs(conv / (n * n) - u).max())
    print(n, worst)
    assert max(worst.values()) <= STEP_TOL, worst


def test_maximum_channels_and_kernels():
    """The largest world the ABI accepts in channels and kernels: C = 16,
    K = 64 (each channel feeds four kernels, outputs spread over all 16)."""
    C, K = 16, 64
    c0 = np.arange(K) % C
    c1 = (np.arange(K) * 5 + 3) % C
    cr = make_creature(32, C, seed=33, c0=c0, c1=c1, radius=(2, 6), seed_box=16)
    check_steps(cr, steps=2)


@pytest.mark.parametrize("trial", range(6))
def test_random_worlds(trial):
    """Seeded random worlds: grid side, channel and kernel counts and the
    c0/c1 maps drawn at random (repeated and unused channels included)."""
    rng = np.random.default_rng(1000 + trial)
    n = int(rng.choice([16, 32, 64, 128]))
    C = int(rng.integers(1, 7))
    K = int(rng.integers(1, 13))
    c0 = rng.integers(0, C, K)
    c1 = rng.integers(0, C, K)
    cr = make_creature(n, C, seed=2000 + trial, c0=c0, c1=c1,
                       radius=(max(2.0, n / 16), max(3.0, n / 5)), seed_box=n // 2,
                       temp=float(rng.uniform(0.5, 2.0)))
    check_steps(cr, steps=2)


def grey_frame(x):
    """The frame the reference's integration test compares
    (train/save_frames_png.py:202-210, ml-rs/save_pngs.rs): the channel sum,
    min-max normalised to 0..255 and truncated to 8 bits."""
    img = x.sum(axis=0).astype(np.float64)
    lo, hi = img.min(), img.max()
    if hi <= lo:
        return np.zeros(img.shape, np.uint8)
    return ((img - lo) / (hi - lo) * 255).astype(np.uint8)


@pytest.mark.parametrize("n", [256, 512])
def test_fifty_steps_within_one_grey_level(n):
    """The reference's acceptance test (scripts/integration.sh:8-46,
    train/compare_pngs.py:72-78): 50 free-running steps, and every frame's
    8-bit grey image within one grey level of the FP64 oracle's."""
    cr = make_creature(n, 3, seed=2024 + n, radius=(n / 40, n / 16), seed_box=n // 2)
    ks = cr.kspec.astype(np.complex128)
    args = (cr.c0, cr.c1, cr.mu.astype(np.float64), cr.sigma.astype(np.float64),
            cr.weights.astype(np.float64), cr.temp)
    x64 = cr.seed.astype(np.float64)
    worst = 0
    with GpuMaceLenia.from_creature(cr) as sim:
        for _ in range(50):
            sim.iterate()
            x64, _, _ = O.step_c(x64, ks, *args, dtype=np.float64, nthreads=os.cpu_count() or 1)
            d = np.abs(grey_frame(sim.state()).astype(int) - grey_frame(x64).astype(int)).max()
            worst = max(worst, int(d))
        drift = float(np.abs(sim.state() - x64).max())
    assert worst <= 1, worst
    assert drift <= 1e-4, drift


@pytest.mark.parametrize("n", [64, 512, 2048])
def test_real_kernel_spectra_path(n):
    """Point-symmetric kernels (every ring kernel here) take the column
    pass's real-spectrum form; a kernel shifted off the origin has a complex
    Hermitian part and keeps the complex form.  Both step like the FP64
    oracle, and the real form agrees with the complex one to rounding."""
    import torch
    cr = make_creature(n, 3, seed=500 + n, radius=(max(2.0, n / 40), max(4.0, n / 16)),
                       seed_box=n // 2)
    a = (cr.kspec.astype(np.complex128), cr.c0, cr.c1, cr.mu.astype(np.float64),
         cr.sigma.astype(np.float64), cr.weights.astype(np.float64), cr.temp)
    with GpuMaceLenia.from_creature(cr) as sim, GpuMaceLenia.from_creature(cr) as cpx:
        assert sim.kernels_real()
        # the same spectra through the device upload keep the complex form
        specs = [torch.tensor(np.stack([cr.kspec[k].real, cr.kspec[k].imag], -1)
                              .astype(np.float32), device="cuda") for k in range(cr.K)]
        torch.cuda.synchronize()        # the uploads, on torch's stream, before cpx reads them
        for k in range(cr.K):
            cpx.set_kernel_device(specs[k].data_ptr(), k)
        cpx.synchronize()
        del specs
        assert not cpx.kernels_real()
        for _ in range(2):
            x = sim.state()
            sim.iterate()
            cpx.iterate()
            ref, _, _ = O.step_c(x.astype(np.float64), *a, nthreads=os.cpu_count() or 1)
            assert np.abs(sim.state() - ref).max() <= STEP_TOL
            # two f32 roundings of the same step (each within the bar above)
            assert np.abs(sim.state() - cpx.state()).max() <= STEP_TOL
    # an asymmetric kernel: kernel 0 shifted by (3, 5) pixels
    shift = np.exp(-2j * np.pi * (3 * np.fft.fftfreq(n)[:, None] + 5 * np.fft.fftfreq(n)[None, :]))
    cr.kspec[0] = (cr.kspec[0] * shift).astype(np.complex64)
    a = (cr.kspec.astype(np.complex128),) + a[1:]
    with GpuMaceLenia.from_creature(cr) as sim:
        assert not sim.kernels_real()
        x = sim.state()
        sim.iterate()
        ref, _, _ = O.step_c(x.astype(np.float64), *a, nthreads=os.cpu_count() or 1)
        assert np.abs(sim.state() - ref).max() <= STEP_TOL


@pytest.mark.parametrize("n", [128, 1024])
def test_graph_layouts_agree(n):
    """Both step-graph layouts (forked channel streams, or one launch per
    phase over all channels) compute the same bits, render graph included."""
    cr = make_creature(n, 3, seed=900 + n, radius=(max(2.0, n / 40), max(4.0, n / 16)),
                       seed_box=n // 2)
    with GpuMaceLenia.from_creature(cr) as a, GpuMaceLenia.from_creature(cr) as b:
        assert a.graph_layout() == 0
        b.set_graph_layout(1)
        assert b.graph_layout() == 1
        a.run_steps(11)
        b.run_steps(11)
        np.testing.assert_array_equal(a.state(), b.state())
        a.iterate_and_render()
        b.iterate_and_render()
        np.testing.assert_array_equal(a.download_render_packed(), b.download_render_packed())
        # the tuner may pick either; tuning does not step the world
        x = b.state()
        b.autotune(reps=2)
        assert b.graph_layout() in (0, 1)
        np.testing.assert_array_equal(b.state(), x)


@pytest.mark.parametrize("var", [[3, 3, 3, 3], [4, 4, 4, 2]])
def test_plan_variants_irregular_and_maximal_maps(var):
    """The FFT-plan variants on the maps that stress the kernel grouping:
    an irregular map at 512^2 (the reference's slot copy mishandles it) and
    the largest world the ABI accepts in channels and kernels (C = 16,
    K = 64), each step against the FP64 oracle."""
    cases = [make_creature(512, 3, seed=61, c0=[1, 0, 2, 1, 2], c1=[0, 1, 1, 2, 0],
                           radius=(8, 30), seed_box=256)]
    C, K = 16, 64
    cases.append(make_creature(512, C, seed=62, c0=np.arange(K) % C, c1=(np.arange(K) * 5 + 3) % C,
                               radius=(8, 24), seed_box=128))
    for cr in cases:
        a = (cr.kspec.astype(np.complex128), cr.c0, cr.c1, cr.mu.astype(np.float64),
             cr.sigma.astype(np.float64), cr.weights.astype(np.float64), cr.temp)
        with GpuMaceLenia.from_creature(cr) as sim:
            sim.set_variants(var)
            for _ in range(2):
                x = sim.state()
                sim.iterate()
                ref, _, _ = O.step_c(x.astype(np.float64), *a, nthreads=os.cpu_count() or 1)
                err = float(np.abs(sim.state() - ref).max())
                assert err <= STEP_TOL, (cr.C, cr.K, err)
