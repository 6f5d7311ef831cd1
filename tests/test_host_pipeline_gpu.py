"""cg_step_host_async: host buffers in and out, pipelined across calls, with
the same results as upload_channel / run_steps / download_all_channels."""
import numpy as np
import pytest

from cella_nova_gb300 import CellaError, GpuMaceLenia
from cella_nova_gb300.creature import make_creature

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def pinned(shape, dtype):
    t = torch.empty(shape, dtype=dtype, pin_memory=True)
    return t, t.numpy()


@pytest.mark.parametrize("n,C", [(64, 2), (256, 3)])
def test_pipelined_steps_match_blocking_path(n, C):
    cr = make_creature(n, C, seed=11, radius=(4, 12) if n == 64 else (8, 30),
                       seed_box=min(n // 2, 256))
    rng = np.random.default_rng(5)
    ins = [rng.random((C, n, n)) for _ in range(4)]
    keep = []
    hin, hout = [], []
    for x in ins:
        ti, ai = pinned((C, n, n), torch.float64)
        to, ao = pinned((C, n, n), torch.float32)
        ai[:] = x
        ao[:] = -1
        keep += [ti, to]
        hin.append(ai)
        hout.append(ao)
    sim = GpuMaceLenia.from_creature(cr)
    twin = GpuMaceLenia.from_creature(cr)
    with sim, twin:
        for i, steps in enumerate((1, 3, 8, 2)):
            sim.step_host_async(hin[i], hout[i], steps)
        sim.host_wait()
        for i, steps in enumerate((1, 3, 8, 2)):
            for c in range(C):
                twin.upload_channel(ins[i][c], c)
            twin.run_steps(steps)
            np.testing.assert_array_equal(hout[i], twin.state())
        # the handle keeps working with the ordinary calls afterwards
        sim.run_steps(2)
        twin.run_steps(2)
        np.testing.assert_array_equal(sim.state(), twin.state())


def test_pageable_buffers_are_rejected():
    cr = make_creature(64, 2, seed=12, radius=(4, 12), seed_box=32)
    with GpuMaceLenia.from_creature(cr) as sim:
        _, ao = pinned((2, 64, 64), torch.float32)
        with pytest.raises(CellaError) as e:
            sim.step_host_async(np.zeros((2, 64, 64)), ao, 1)
        assert e.value.code == -1
        sim.run_steps(1)
        assert np.isfinite(sim.state()).all()
