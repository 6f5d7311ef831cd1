"""Render (iterate_and_render, render, download_render) and the
device-resident growth parameters, through the C ABI."""
import numpy as np
import pytest

from cella_nova_gb300 import GpuMaceLenia
from cella_nova_gb300.creature import make_creature
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,C", [(64, 1), (64, 2), (128, 3), (64, 4), (256, 3)])
def test_iterate_and_render_matches_oracle_render(n, C):
    cr = make_creature(n, C, seed=30 + C, radius=(max(2.0, n / 16), max(4.0, n / 6)),
                       seed_box=n // 2)
    with GpuMaceLenia.from_creature(cr) as a, GpuMaceLenia.from_creature(cr) as b:
        assert (a.download_render_packed() == 0).all()      # zeros until the first render
        for _ in range(3):
            a.iterate_and_render()
            b.iterate()
            x = a.state()
            np.testing.assert_array_equal(x, b.state())    # rendering does not change the step
            packed = a.download_render_packed()
            np.testing.assert_array_equal(packed, O.render_np(x))
        np.testing.assert_array_equal(a.download_render(), O.rgb24_np(packed))
        # the standalone render of the same state gives the same words
        b.render()
        np.testing.assert_array_equal(b.download_render_packed(), packed)
        # graph steps afterwards leave the render buffer alone
        a.run_steps(9)
        np.testing.assert_array_equal(a.download_render_packed(), packed)


@pytest.mark.parametrize("n,C", [(64, 3), (256, 2), (512, 3)])
def test_render_levels_in_every_diffusion_variant(n, C):
    """A rendering step's level bytes come from whichever diffusion body the
    world runs (one byte, two or four per store): every variant gives the
    oracle's words and the same state as a plain step."""
    cr = make_creature(n, C, seed=60 + n, radius=(max(2.0, n / 16), max(4.0, n / 6)),
                       seed_box=n // 2)
    for v in range(4):
        with GpuMaceLenia.from_creature(cr) as a, GpuMaceLenia.from_creature(cr) as b:
            a.set_variants([0, 0, 0, v])
            b.set_variants([0, 0, 0, v])
            for _ in range(2):
                a.iterate_and_render()
                b.iterate()
            x = a.state()
            np.testing.assert_array_equal(x, b.state(), err_msg=f"diffusion variant {v}")
            np.testing.assert_array_equal(a.download_render_packed(), O.render_np(x),
                                          err_msg=f"diffusion variant {v}")


def test_render_saturates_and_clamps():
    n, C = 64, 3
    cr = make_creature(n, C, seed=5, radius=(4, 10), seed_box=32)
    with GpuMaceLenia.from_creature(cr) as sim:
        x = np.zeros((C, n, n), np.float64)
        x[0, :, : n // 2] = 5.0
        x[1] = np.linspace(-1, 1, n * n).reshape(n, n)
        x[2, n // 2:] = 0.3
        sim.upload_state(x)
        sim.render()
        got = sim.download_render_packed()
        np.testing.assert_array_equal(got, O.render_np(x.astype(np.float32)))


def test_set_params_takes_effect_without_changing_other_steps():
    """New parameters reach the captured graphs (device-resident block): a
    world whose parameters were replaced steps exactly like a world created
    with them."""
    cr = make_creature(128, 3, seed=40, radius=(8, 20), seed_box=64)
    cr2 = make_creature(128, 3, seed=41, radius=(8, 20), seed_box=64)
    with GpuMaceLenia.from_creature(cr) as a:
        a.run_steps(2)
        x = a.state()
        a.set_params(cr2.mu, cr2.sigma, cr2.weights, cr.temp)
        a.run_steps(9)
        got = a.state()
    with GpuMaceLenia((128, 128), 3, cr.K, cr.c0, cr.c1, cr2.mu, cr2.sigma, cr2.weights,
                      cr.temp) as b:
        for k in range(cr.K):
            b.set_kernel(cr.kspec[k], k)
        b.upload_state(x)
        b.run_steps(9)
        np.testing.assert_array_equal(got, b.state())


def test_set_params_device_equals_host_folding():
    import torch
    cr = make_creature(128, 3, seed=42, radius=(8, 20), seed_box=64)
    cr2 = make_creature(128, 3, seed=43, radius=(8, 20), seed_box=64)
    dev = [torch.tensor(np.asarray(v, np.float32), device="cuda")
           for v in (cr2.mu, cr2.sigma, cr2.weights)]
    torch.cuda.synchronize()
    with GpuMaceLenia.from_creature(cr) as a, GpuMaceLenia.from_creature(cr) as b:
        a.set_params(cr2.mu, cr2.sigma, cr2.weights, cr.temp)
        b.set_params_device(*[t.data_ptr() for t in dev])
        a.run_steps(5)
        b.run_steps(5)
        np.testing.assert_array_equal(a.state(), b.state())


def test_stream_frames_to_a_file_and_a_pipe(tmp_path):
    """Frame streaming writes exactly the frames the iterate_and_render +
    download_render loop of main.rs produces, to a file or through a pipe."""
    import os
    import threading
    n, frames, spf = 64, 5, 2
    cr = make_creature(n, 3, seed=21, radius=(4, 12), seed_box=32)
    with GpuMaceLenia.from_creature(cr) as a, GpuMaceLenia.from_creature(cr) as b, \
            GpuMaceLenia.from_creature(cr) as c:
        path = tmp_path / "frames.rgb"
        with open(path, "wb") as f:
            a.stream_frames(f.fileno(), frames, steps_per_frame=spf)
        raw = np.fromfile(path, np.uint8).reshape(frames, n, n, 3)
        for i in range(frames):
            b.run_steps(spf - 1)
            b.iterate_and_render()
            np.testing.assert_array_equal(raw[i], b.download_render(), err_msg=f"frame {i}")
        np.testing.assert_array_equal(a.state(), b.state())
        # the same through a pipe, read by another thread (as an encoder would)
        rfd, wfd = os.pipe()
        got = []

        def reader():
            with os.fdopen(rfd, "rb") as r:
                got.append(r.read())

        th = threading.Thread(target=reader)
        th.start()
        c.stream_frames(wfd, frames, steps_per_frame=spf)
        os.close(wfd)
        th.join(timeout=60)
        np.testing.assert_array_equal(np.frombuffer(got[0], np.uint8).reshape(frames, n, n, 3), raw)
