"""Golden fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py):
the oracle must reproduce them bit for bit on the CPU, and the device hider
must match them on the GPU at the parity bars (winners, occluding depths,
fragment counts and valid flags bit-exact; filtered channels within 1e-5
relative; quantized values within 1 LSB)."""
import glob
import os

import numpy as np
import pytest

from aqsis_gb300 import scene as S

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
NAMES = [os.path.splitext(os.path.basename(p))[0] for p in FIXTURES]
OUT_KEYS = ("winner", "occlz", "nfrag", "valid", "channels", "quantized")


def test_fixtures_present():
    assert len(FIXTURES) >= 23


@pytest.mark.parametrize("path", FIXTURES, ids=NAMES)
def test_oracle_reproduces_fixture(oracle, path):
    sc, gold = S.load_scene(path)
    res = oracle.render(sc, tuple(int(c) for c in gold["qchannels"]))
    for k in OUT_KEYS + (("aov",) if "o_aov" in gold else ()):
        a, b = np.asarray(res[k]), gold["o_" + k]
        assert a.shape == b.shape, k
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), "%s differs" % k


@pytest.mark.parametrize("path", FIXTURES[:3], ids=NAMES[:3])
def test_scene_file_round_trip(path, tmp_path):
    sc, gold = S.load_scene(path)
    out = tmp_path / "copy.npz"
    S.save_scene(str(out), sc)
    sc2, _ = S.load_scene(str(out))
    assert sc2.frame == sc.frame
    for k in ("cu", "cv", "P", "Ci", "Oi", "flags", "pbase", "cbase"):
        assert np.array_equal(getattr(sc.grids, k), getattr(sc2.grids, k))
    assert np.array_equal(sc.samples.pos, sc2.samples.pos)


def test_fixtures_cover_the_hider_features():
    feats = set()
    for p in FIXTURES:
        sc, gold = S.load_scene(p)
        fr, g = sc.frame, sc.grids
        if fr.shutter[1] != fr.shutter[0]:
            feats.add("motion")
        if fr.use_dof:
            feats.add("dof")
        if not (g.flags & S.GRID_OPAQUE).all():
            feats.add("transparent")
        if (g.flags & S.GRID_MATTE).any():
            feats.add("matte")
        if g.culled is not None:
            feats.add("culled")
        if fr.crop is not None:
            feats.add("crop")
        if fr.depth_filter:
            feats.add("depth_filter_%d" % fr.depth_filter)
        if fr.q_dither:
            feats.add("dither")
        if (g.flags & S.GRID_TRIANGULAR).any():
            feats.add("triangular")
        if (g.flags & S.GRID_CAMERA).any() and fr.camera_to_raster is not None:
            feats.add("camera_space")
        if g.aov is not None and "o_aov" in gold:
            feats.add("output_variables")
        feats.add("filter_" + fr.filter)
        assert gold["o_valid"].any()
    for f in ("motion", "dof", "transparent", "matte", "culled", "crop", "dither", "depth_filter_1",
              "depth_filter_2", "depth_filter_3", "filter_box", "filter_gaussian", "filter_catmull-rom", "triangular",
              "camera_space", "output_variables"):
        assert f in feats, f


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=NAMES)
def test_device_matches_fixture(hider, path):
    from tests.test_gpu_parity import close_or_same
    sc, gold = S.load_scene(path)
    res = hider.render_scene(sc, tuple(int(c) for c in gold["qchannels"]))
    for k in ("winner", "nfrag", "valid"):
        assert np.array_equal(res[k], gold["o_" + k]), k
    assert np.array_equal(res["occlz"].view(np.uint32), gold["o_occlz"].view(np.uint32))
    ok = close_or_same(res["channels"], gold["o_channels"])
    assert ok.all(), "channels differ at %d entries" % int((~ok).sum())
    q = np.abs(res["quantized"].astype(np.int64) - gold["o_quantized"].astype(np.int64))
    assert q.max() <= 1
    if "o_aov" in gold:
        ok = close_or_same(res["aov"], gold["o_aov"])
        assert ok.all(), "output variables differ at %d entries" % int((~ok).sum())
