"""Imager shaders through the C-ABI: aqh_set_imager stops the frame after
the filter, the channels read back are FilterBucket's (before exposure), a
host-side stand-in for the imager shader computes new colours and
opacities from them, and aqh_apply_imager writes them back, sets alpha and
applies exposure and the 8-bit display.  Checked against the oracle's
restatement of bucketprocessor.cpp:712-743 and ExposeBucket, in both
execution forms, bit-exact channels and 8-bit values within 1 LSB."""
import dataclasses

import numpy as np
import pytest

from tests import scenes_small as SS
from tests.test_gpu_parity import close_or_same

pytestmark = pytest.mark.gpu


def _scene(seed, transparent=False):
    from aqsis_gb300 import scene as S
    sc = SS.transparent_small(seed=seed) if transparent else SS.edge_cases(seed=seed)
    sc.frame.crop = (3, sc.frame.width - 2, 2, sc.frame.height - 1)
    sc.frame.gain, sc.frame.gamma = 1.7, 2.2
    sc.frame.q_dither = 0.5
    sc.samples = S.make_samples(sc.frame, np.random.default_rng(seed), 32, dither=True)
    return sc


def _shader(pre):
    """A stand-in for an imager shader run by the host's shading VM: a
    function of each pixel's filtered colour, opacity and depth."""
    ci, oi = pre[..., 0:3], pre[..., 3:6]
    out = np.empty(pre.shape[:-1] + (6,), np.float32)
    out[..., 0:3] = np.float32(1.0) - ci * np.float32(0.75)
    out[..., 3:6] = oi * np.float32(0.5) + np.float32(0.25)
    return out


@pytest.mark.parametrize("batched", [False, True], ids=["plain", "batched"])
@pytest.mark.parametrize("transparent", [False, True], ids=["opaque", "transparent"])
def test_imager_write_back(aqh_lib, oracle, batched, transparent):
    sc = _scene(301 + transparent, transparent)
    h = aqh_lib.Hider(0)
    try:
        h.set_mode(batched)
        h.set_imager(True)
        h.frame_begin(sc.frame)
        h.set_samples(sc.samples)
        h.submit_scene_grids(sc.grids)
        h.render(sync=True)
        pre = h.read_channels()
        im = _shader(pre)
        h.apply_imager(im)
        post = h.read_channels()
        q = h.read_quantized((0, 1, 2, 6))
    finally:
        h.close()
    # the oracle's filter output before exposure, then the imager and exposure
    raw = dataclasses.replace(sc.frame, gain=1.0, gamma=1.0)
    ref_pre = oracle.render(type(sc)(raw, sc.grids, sc.samples), want_samples=False)["channels"]
    assert close_or_same(pre, ref_pre).all()
    assert transparent or np.array_equal(pre.view(np.uint32), ref_pre.view(np.uint32))
    ref_post = oracle.imager(sc.frame, ref_pre, _shader(ref_pre))
    ok = close_or_same(post, ref_post)
    assert ok.all(), "channels differ at %d entries" % int((~ok).sum())
    ref_q = oracle.quantize(sc.frame, ref_post, sc.samples.dither)
    assert np.abs(q.astype(np.int64) - ref_q.astype(np.int64)).max() <= 1


def test_apply_without_an_imager_frame_is_refused(aqh_lib):
    sc = _scene(311)
    h = aqh_lib.Hider(0)
    try:
        h.frame_begin(sc.frame)
        h.set_samples(sc.samples)
        h.submit_scene_grids(sc.grids)
        h.render(sync=True)
        with pytest.raises(aqh_lib.AqhError):
            h.apply_imager(np.zeros((1, 6), np.float32))
    finally:
        h.close()
