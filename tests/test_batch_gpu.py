"""Batched worlds (persistent launch per phase) against single worlds and the
FP64 oracle, through the C ABI."""
import numpy as np
import pytest

from cella_nova_gb300 import GpuMaceLenia, GpuMaceLeniaBatch
from cella_nova_gb300.creature import all_pairs, make_creature
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def mixed_creatures():
    rng = np.random.default_rng(7)
    out = []
    for i, (n, C) in enumerate([(256, 3), (64, 1), (128, 4), (256, 2), (64, 3), (512, 2)]):
        out.append(make_creature(n, C, seed=300 + i, radius=(max(2.0, n / 16), max(4.0, n / 6)),
                                 seed_box=n // 2, temp=float(rng.uniform(0.5, 2.0))))
    return out


def test_batched_worlds_equal_single_worlds():
    crs = mixed_creatures()
    with GpuMaceLeniaBatch(crs) as b:
        b.run_steps(3)
        b.synchronize()
        for i, cr in enumerate(crs):
            with GpuMaceLenia.from_creature(cr) as s:
                s.run_steps(3)
                np.testing.assert_array_equal(b.state(i), s.state(), err_msg=f"world {i}")


def test_batched_step_parity_with_oracle():
    crs = mixed_creatures()
    with GpuMaceLeniaBatch(crs) as b:
        b.run_steps(2)
        xs = [b.state(i) for i in range(len(crs))]
        b.run_steps(1)
        for i, cr in enumerate(crs):
            ref, _, _ = O.step_c(xs[i].astype(np.float64), cr.kspec.astype(np.complex128),
                                 cr.c0, cr.c1, cr.mu.astype(np.float64),
                                 cr.sigma.astype(np.float64), cr.weights.astype(np.float64),
                                 cr.temp) if cr.n <= 256 else O.step_np(
                xs[i].astype(np.float64), cr.kspec.astype(np.complex128), cr.c0, cr.c1,
                cr.mu.astype(np.float64), cr.sigma.astype(np.float64),
                cr.weights.astype(np.float64), cr.temp)
            assert np.abs(b.state(i) - ref).max() <= 1e-5, i


def test_batched_mass_and_info():
    crs = mixed_creatures()
    with GpuMaceLeniaBatch(crs) as b:
        m0 = [b.mass_f64(i) for i in range(len(crs))]
        b.run_steps(50)
        for i in range(len(crs)):
            assert np.abs(b.mass_f64(i) / m0[i] - 1).max() < 1e-6
        items, grid = b.info()
        assert all(x > 0 for x in items) and all(g > 0 for g in grid)


def test_batch_rejects_bad_world():
    from cella_nova_gb300 import CellaError
    cr = make_creature(32, 1, seed=1, radius=(2, 4), seed_box=16)
    with pytest.raises(CellaError, match="world 0"):
        GpuMaceLeniaBatch([cr])


def test_batch_autotune_keeps_the_results():
    """The batch's autotuner picks per grid side among the variants that
    side has (CTA shapes that agree bit for bit; from 512 on also FFT plans
    that agree to rounding) and does not step the worlds."""
    crs = mixed_creatures()
    with GpuMaceLeniaBatch(crs) as a, GpuMaceLeniaBatch(crs) as b:
        x0 = [b.state(i) for i in range(len(crs))]
        tuned = b.autotune(reps=2)
        assert sorted(tuned) == sorted({cr.n for cr in crs})
        for side, (chosen, ms) in tuned.items():
            counts = [4 if p == 3 else (5 if side >= 512 else 3) for p in range(4)]
            assert ms.shape == (4, 5)
            for p in range(4):
                assert 0 <= chosen[p] < counts[p]
                assert (ms[p, :counts[p]] > 0).all() and (ms[p, counts[p]:] == -1).all()
        for i in range(len(crs)):
            np.testing.assert_array_equal(b.state(i), x0[i])
        a.run_steps(4)
        b.run_steps(4)
        for i, cr in enumerate(crs):
            if max(tuned[cr.n][0][:3]) <= 2:
                np.testing.assert_array_equal(b.state(i), a.state(i), err_msg=str(i))
            else:
                assert np.abs(b.state(i) - a.state(i)).max() <= 4e-5, i


def test_batched_plan_variants_match_single_worlds():
    """The batch's FFT-plan variants and its streaming forward row pass and
    8-row diffusion strips (at 512^2) step like the single-world kernels of
    the same variants, bit for bit."""
    crs = [make_creature(512, 2, seed=410, temp=1.2), make_creature(512, 3, seed=411)]
    for var in ([2, 2, 2, 3], [3, 3, 3, 3], [4, 4, 4, 2]):
        with GpuMaceLeniaBatch(crs) as b:
            b.set_variants(512, var)
            b.run_steps(3)
            for i, cr in enumerate(crs):
                with GpuMaceLenia.from_creature(cr) as s:
                    s.set_variants(var)
                    s.run_steps(3)
                    np.testing.assert_array_equal(b.state(i), s.state(), err_msg=f"{var} {i}")


def test_batch_world_branch_mode_equals_single_worlds():
    """Mode 1 (each world's own step kernels, the worlds as parallel graph
    branches) steps every world exactly like a single world with the same
    variants, as mode 0 does."""
    crs = mixed_creatures()
    with GpuMaceLeniaBatch(crs) as b:
        for side in sorted({cr.n for cr in crs}):
            b.set_mode(side, 1)
            assert b.mode(side) == 1
        b.run_steps(3)
        for i, cr in enumerate(crs):
            with GpuMaceLenia.from_creature(cr) as s:
                s.run_steps(3)
                np.testing.assert_array_equal(b.state(i), s.state(), err_msg=f"world {i}")
        # back to persistent launches, mid-run
        b.set_mode(512, 0)
        b.run_steps(2)
        with GpuMaceLenia.from_creature(crs[5]) as s:
            s.run_steps(5)
            np.testing.assert_array_equal(b.state(5), s.state())
