"""Display requests (aqh_read_display): FormatBucketForDisplay's quantize and
element-type conversion for every Dspy type, checked against the oracle's
quantized values for the same request settings."""
import dataclasses

import numpy as np
import pytest

from aqsis_gb300 import aqh as A
from tests import scenes_small as SS

pytestmark = pytest.mark.gpu

REQUESTS = [
    # channels, one, min, max, dither
    ((6, 0, 1, 2), 255.0, 0.0, 255.0, 0.5),        # rgba, 8-bit unsigned
    ((0, 1, 2), 65535.0, 0.0, 65535.0, 0.5),        # 16-bit unsigned
    ((0, 3), 1.0e6, 0.0, 4.0e9, 0.0),               # 32-bit unsigned
    ((0, 1), 100.0, -128.0, 127.0, 0.5),            # 8-bit signed
    ((2, 6), 20000.0, -32768.0, 32767.0, 1.0),      # 16-bit signed
    ((0, 8), 3.0e6, -5.0e6, 5.0e6, 0.0),            # 32-bit signed
    ((7,), 0.0, 0.0, 0.0, 0.0),                     # z, unquantized float
    ((6, 0), 250.0, 2.0, 240.5, 0.25),              # clamped to a non-integral max
]


def as_type(v, fmt):
    """ddmanager.cpp:1069-1113: 32-bit integers clamped to their range, then a C conversion."""
    dt = A.DSPY_DTYPES[fmt]
    if fmt == 2:
        v = np.clip(v, 0, 4294967295.0)
    elif fmt == 3:
        v = np.clip(v, -2147483648.0, 2147483647.0)
    if fmt == 1:
        return v.astype(np.float32)
    return np.trunc(v).astype(np.int64).astype(dt)


@pytest.mark.parametrize("req", REQUESTS, ids=[str(r[1]) + "_" + str(r[2]) for r in REQUESTS])
def test_display_request_matches_oracle(hider, oracle, req):
    ch, one, lo, hi, damp = req
    sc = SS.opaque_small(seed=51, scale=0.03)
    rng = np.random.default_rng(5)
    cx0, cx1, cy0, cy1 = sc.frame.crop_window
    dither = rng.random((cy1 - cy0) * (cx1 - cx0)).astype(np.float32)
    hider.render_scene(sc, samples=False)
    got = hider.read_display(ch, one=one, qmin=lo, qmax=hi, dither_amp=damp, dither=dither)
    fmt = hider.L.aqh_display_format(one, lo, hi)
    fr = dataclasses.replace(sc.frame, q_one=one, q_min=lo, q_max=hi, q_dither=damp)
    ref_sc = type(sc)(fr, sc.grids, dataclasses.replace(sc.samples, dither=dither))
    ref = oracle.render(ref_sc, ch, want_samples=False)
    want = as_type(np.asarray(ref["quantized"], np.float64).reshape(got.shape), fmt)
    assert got.dtype == want.dtype
    if fmt == 1:
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)) or \
            np.array_equal(got, want, equal_nan=True)
    else:
        assert np.array_equal(got, want), "differs at %d values" % int((got != want).sum())


def test_u8_request_equals_fused_quantize(hider):
    sc = SS.opaque_small(seed=52, scale=0.03)
    res = hider.render_scene(sc, samples=False)
    f = sc.frame
    got = hider.read_display((0, 1, 2, 6), one=f.q_one, qmin=f.q_min, qmax=f.q_max, dither_amp=f.q_dither)
    assert np.array_equal(got, res["quantized"])


def test_rendered_frame_to_capture_driver(hider, tmp_path):
    """aqh_dspy_send: the request read from the device and delivered to the
    capture driver in buckets equals the fused 8-bit quantize."""
    from tests.test_dspy import read_ppm
    sc = SS.opaque_small(seed=53, scale=0.03)
    res = hider.render_scene(sc, samples=False)
    path = str(tmp_path / "frame.ppm")
    f = sc.frame
    dd = A.DisplayDriver(A.capture_driver_path(), path, hider.dspy_geometry(), (6, 0, 1, 2), ["a", "r", "g", "b"],
                         one=f.q_one, qmin=f.q_min, qmax=f.q_max, dither_amp=f.q_dither)
    dd.send(hider)
    dd.close()
    assert np.array_equal(read_ppm(path), res["quantized"][..., :3])
