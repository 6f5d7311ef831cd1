"""Error returns of the C ABI on a live handle: the call fails with its
status code and leaves the world usable."""
import numpy as np
import pytest

from cella_nova_gb300 import CellaError, GpuMaceLenia
from cella_nova_gb300.creature import make_creature
from cella_nova_gb300.orchestrator import creature_ring_specs

pytestmark = pytest.mark.gpu

ARG, IO = -1, -5


def world(seed=3):
    cr = make_creature(64, 2, seed=seed, radius=(4, 12), seed_box=32)
    return cr, GpuMaceLenia.from_creature(cr)


def assert_code(code, fn, *args, **kw):
    with pytest.raises(CellaError) as e:
        fn(*args, **kw)
    assert e.value.code == code, e.value


def test_bad_ring_specs_are_rejected():
    cr, sim = world()
    with sim:
        specs, _ = creature_ring_specs(cr)
        bad_family = [(5, 1, 8.0, 0.0)] + specs[1:]
        too_many = [(0, 9, 8.0, 0.0)] + specs[1:]
        no_radius = [(0, 1, 0.0, 0.0)] + specs[1:]
        no_width = [(1, 1, 8.0, 0.0)] + specs[1:]
        for bad in (bad_family, too_many, no_radius, no_width):
            assert_code(ARG, sim.build_ring_kernels, bad)
        x = sim.state()
        sim.iterate()    # still steps
        assert np.isfinite(sim.state()).all() and not np.array_equal(sim.state(), x)


def test_frame_stream_to_an_invalid_descriptor_fails_cleanly():
    cr, sim = world(4)
    with sim:
        assert_code(ARG, sim.stream_frames, -1, 2)
        # a descriptor number far above any open one: write() fails (EBADF)
        assert_code(IO, sim.stream_frames, 1 << 20, 2)
        sim.run_steps(3)    # the world keeps stepping
        assert np.isfinite(sim.state()).all()


def test_parameter_and_variant_errors_leave_the_world_unchanged():
    cr, sim = world(5)
    _, twin = world(5)
    with sim, twin:
        bad_sigma = np.asarray(cr.sigma, np.float32).copy()
        bad_sigma[0] = np.nan
        assert_code(ARG, sim.set_params, cr.mu, bad_sigma, cr.weights)
        assert_code(ARG, sim.set_variants, [0, 3, 0, 0])
        sim.run_steps(4)
        twin.run_steps(4)
        np.testing.assert_array_equal(sim.state(), twin.state())


def test_unroll_argument_errors():
    import ctypes
    torch = pytest.importorskip("torch")
    from cella_nova_gb300.autograd import LeniaWorld
    cr = make_creature(64, 2, seed=6, radius=(4, 12), seed_box=32)
    w = LeniaWorld(cr.n, cr.C, cr.c0, cr.c1, cr.temp)
    x = torch.zeros((cr.C, 64, 64), device="cuda")
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    assert w.lib.cg_unroll(w.h, P(x), 0, 4, P(x), P(x)) == ARG
    assert w.lib.cg_unroll(w.h, P(x), 4, 0, P(x), P(x)) == ARG
    assert w.lib.cg_unroll(w.h, None, 4, 4, P(x), P(x)) == ARG
    w.close()


def test_misaligned_device_buffers_are_rejected():
    """Device buffers start on 16-byte boundaries (the kernels read them with
    16-byte loads and bulk copies): a pointer 4 bytes in is refused on the
    host, before anything is launched, and the world still steps."""
    import ctypes
    torch = pytest.importorskip("torch")
    from cella_nova_gb300.autograd import LeniaWorld
    cr = make_creature(64, 2, seed=6, radius=(4, 12), seed_box=32)
    w = LeniaWorld(cr.n, cr.C, cr.c0, cr.c1, cr.temp)
    plane = cr.C * 64 * 64
    buf = torch.zeros(2 * plane + 8, device="cuda")
    x, y = buf[:plane], buf[plane + 4:2 * plane + 4]
    odd = ctypes.c_void_p(buf.data_ptr() + 4)
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    assert w.lib.cg_step_from(w.h, odd, P(y)) == ARG
    assert b"16-byte aligned" in w.lib.cg_last_error()
    assert w.lib.cg_step_from(w.h, P(x), odd) == ARG
    assert w.lib.cg_unroll(w.h, odd, 4, 4, P(y), P(x)) == ARG
    assert w.lib.cg_set_kernel_device(w.h, 0, odd) == ARG
    assert w.lib.cg_step_from(w.h, P(x), P(y)) == 0
    torch.cuda.synchronize()
    assert torch.isfinite(y).all()
    w.close()


def test_bounded_wait_gives_up_and_reports_timeout():
    """A device-side wait that nothing completes (an mbarrier no thread or
    copy arrives on) ends at its limit with the timeout status; the context
    and the handle stay usable, and the world steps exactly as its twin."""
    TIMEOUT = -4
    cr, sim = world(7)
    _, twin = world(7)
    with sim, twin:
        sim.run_steps(2)
        twin.run_steps(2)
        for ms in (5, 50):
            assert_code(TIMEOUT, sim.check_bounded_wait, ms)
        assert_code(ARG, sim.check_bounded_wait, 0)
        assert_code(ARG, sim.check_bounded_wait, 5000)
        sim.run_steps(3)      # the error word was cleared: steps report OK
        twin.run_steps(3)
        np.testing.assert_array_equal(sim.state(), twin.state())
