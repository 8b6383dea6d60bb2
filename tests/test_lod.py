"""Level of detail in the oracle: a grid's LevelOfDetailBounds [min, max)
keep it from samples whose detail level lies outside (a min below 0 turns
the test off; the default 0 1 passes every level in [0, 1))."""
import dataclasses

import numpy as np
import pytest

from aqsis_gb300 import scene as S
from tests import scenes_small as SS


def lod_scene(bounds, seed=3):
    fr = S.Frame(width=8, height=8, xsamples=2, ysamples=2, filter="box", xfilter=1.0, yfilter=1.0, q_dither=0.0)
    g = SS.plane(0, 0, 8, 8, 2.0, flags=S.GRID_SMOOTH)
    g.lod = np.array([bounds], np.float32)
    sc = SS.custom(fr, g, seed=seed, explicit=True)
    rng = np.random.default_rng(seed)
    lod = rng.random(np.asarray(sc.samples.pos).reshape(-1, 2).shape[0]).astype(np.float32)
    return S.Scene(sc.frame, sc.grids, dataclasses.replace(sc.samples, lod=lod)), lod


@pytest.mark.parametrize("bounds", [(0.5, 1.0), (0.0, 0.25), (0.3, 0.6), (-1.0, 0.0), (0.0, 1.0)])
def test_detail_bounds_select_samples(oracle, bounds):
    sc, lod = lod_scene(bounds)
    res = oracle.render(sc)
    hit = res["winner"] >= 0
    x0, y0, w, h = sc.frame.sample_region
    spp = sc.frame.spp
    # samples of the image's own pixels all lie inside the plane
    inside = np.zeros((h, w, spp), bool)
    inside[1:-1, 1:-1] = True
    inside = inside.reshape(-1)
    if bounds[0] < 0:
        want = np.ones_like(lod, bool)
    else:
        want = (lod >= bounds[0]) & (lod < bounds[1])
    assert np.array_equal(hit[inside], want[inside])


def test_scene_file_keeps_detail_bounds(tmp_path):
    sc, _ = lod_scene((0.2, 0.7))
    p = tmp_path / "lod.npz"
    S.save_scene(str(p), sc)
    sc2, _ = S.load_scene(str(p))
    assert np.array_equal(sc2.grids.lod, sc.grids.lod)
    assert np.array_equal(sc2.samples.lod, sc.samples.lod)
