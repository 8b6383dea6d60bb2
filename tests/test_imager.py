"""Imager shaders, oracle side: the write-back of bucketprocessor.cpp:712-743
(Ci and Oi from the shader, alpha = the mean of that opacity, no coverage
factor) followed by ExposeBucket (766-806), checked on hand-made values."""
import numpy as np

from aqsis_gb300 import scene as S


def test_imager_write_back_and_exposure(oracle):
    fr = S.Frame(width=2, height=1, gain=2.0, gamma=1.0)
    chan = np.zeros((1, 2, 9), np.float32)
    chan[..., 7] = [5.0, 7.0]          # depth and coverage are kept
    chan[..., 8] = [0.25, 1.0]
    im = np.array([[0.1, 0.2, 0.3, 0.5, 0.25, 1.0],
                   [1.0, 0.0, 0.5, 0.0, 0.0, 0.0]], np.float32)
    out = oracle.imager(fr, chan, im)
    np.testing.assert_array_equal(out[0, :, 0:3], im[:, 0:3] * np.float32(2.0))
    np.testing.assert_array_equal(out[0, :, 3:6], im[:, 3:6])
    a = ((im[:, 3] + im[:, 4]) + im[:, 5]) / np.float32(3.0)
    np.testing.assert_array_equal(out[0, :, 6], a)
    np.testing.assert_array_equal(out[0, :, 7], [5.0, 7.0])
    np.testing.assert_array_equal(out[0, :, 8], [0.25, 1.0])


def test_imager_gamma_and_quantize(oracle):
    fr = S.Frame(width=1, height=1, gain=1.0, gamma=2.0, q_dither=0.0)
    chan = np.zeros((1, 1, 9), np.float32)
    im = np.array([[0.25, 0.0, 1.0, 1.0, 1.0, 1.0]], np.float32)
    out = oracle.imager(fr, chan, im)
    np.testing.assert_allclose(out[0, 0, 0:3], [0.5, 0.0, 1.0], rtol=1e-7)
    q = oracle.quantize(fr, out)
    # round(0.5 * 255) = 128 (lround rounds halves up), alpha 1 -> 255
    np.testing.assert_array_equal(q[0, 0], [128, 0, 255, 255])
