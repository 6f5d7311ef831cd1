"""The render restatement (CPU): known answers of render_main
(ml-rs/shaders/compute_1024.wgsl:428-443) worked by hand."""
import numpy as np

from oracle import oracle as O


def test_levels_known_answers():
    # level = u32(sqrt(clamp(1.5 c, 0, 1)) * 255), f32 throughout
    c = np.array([0.0, 0.1, 0.5, 2.0 / 3.0, 1.0, 5.0, -0.3, np.nan, 1e-6], np.float32)
    want = np.array([0, 98, 220, 255, 255, 255, 0, 0, 0], np.uint32)
    got = O.render_np(c[None, None, :])[0] >> 16
    np.testing.assert_array_equal(got, want)


def test_packing_and_missing_channels():
    x = np.zeros((4, 2, 2), np.float32)
    x[0, 0, 0] = 1.0     # R
    x[1, 0, 1] = 1.0     # G
    x[2, 1, 0] = 1.0     # B
    x[3] = 1.0           # a fourth channel is not drawn
    p = O.render_np(x)
    np.testing.assert_array_equal(p, [[0xFF0000, 0x00FF00], [0x0000FF, 0]])
    np.testing.assert_array_equal(O.render_np(x[:1]), [[0xFF0000, 0], [0, 0]])
    np.testing.assert_array_equal(O.render_np(x[:2]), [[0xFF0000, 0x00FF00], [0, 0]])


def test_rgb24_bytes():
    p = np.array([[0x123456, 0xABCDEF]], np.uint32)
    np.testing.assert_array_equal(O.rgb24_np(p), [[[0x12, 0x34, 0x56], [0xAB, 0xCD, 0xEF]]])
