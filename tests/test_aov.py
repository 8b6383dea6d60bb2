"""Output variables in the oracle: each sample carries the vertex-A values of
its front hit (StoreExtraData + Combine), averaged by the pixel filter."""
import dataclasses

import numpy as np
import pytest

from aqsis_gb300 import scene as S
from tests import scenes_small as SS


def two_planes(near_oi=None, order=("near", "far")):
    """8x8 image, 2x2 samples, box 1x1: a far opaque plane (z 5, output
    variables 7, -3) and a near plane (z 2) whose vertex (i, j) carries
    (i + 10 j, -j); both planes have one micropolygon per pixel."""
    fr = S.Frame(width=8, height=8, xsamples=2, ysamples=2, filter="box", xfilter=1.0, yfilter=1.0, q_dither=0.0)
    near = SS.plane(0, 0, 8, 8, 2.0, oi=near_oi, flags=0)
    far = SS.plane(0, 0, 8, 8, 5.0, flags=0)
    jj, ii = np.divmod(np.arange(81), 9)
    near.aov = np.stack([ii + 10 * jj, -jj], -1).astype(np.float32)
    far.aov = np.tile(np.array([[7.0, -3.0]], np.float32), (81, 1))
    parts = [near, far] if order[0] == "near" else [far, near]
    g = S.concat_grids(parts)
    g.aov = np.concatenate([p.aov for p in parts])
    return SS.custom(fr, g, seed=3)


@pytest.mark.parametrize("order", [("near", "far"), ("far", "near")])
def test_opaque_front_vertex_a_values(oracle, order):
    res = oracle.render(two_planes(order=order))
    a = res["aov"]
    y, x = np.mgrid[0:8, 0:8]
    assert np.array_equal(a[..., 0], (x + 10 * y).astype(np.float32))
    assert np.array_equal(a[..., 1], (-y).astype(np.float32))


def test_transparent_front_fragment_values(oracle):
    res = oracle.render(two_planes(near_oi=np.full((81, 3), 0.5)))
    y, x = np.mgrid[0:8, 0:8]
    assert np.array_equal(res["aov"][..., 0], (x + 10 * y).astype(np.float32))
    # the far plane's colour shows through, but the output variables are the front's
    assert (res["channels"][..., 0] > 0).all()


def test_no_hits_give_zero(oracle):
    sc = two_planes()
    sc.frame = dataclasses.replace(sc.frame, width=12)     # columns 8..11 see nothing
    sc = SS.custom(sc.frame, sc.grids, seed=3)
    res = oracle.render(sc)
    assert (res["aov"][:, 9:] == 0).all()


def test_scene_file_keeps_output_variables(tmp_path):
    sc = S.with_aov(SS.edge_cases(seed=3), 3, 5)
    p = tmp_path / "aov.npz"
    S.save_scene(str(p), sc)
    sc2, _ = S.load_scene(str(p))
    assert np.array_equal(sc2.grids.aov, sc.grids.aov)
