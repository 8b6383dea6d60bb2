"""Trim curves in the oracle (Split's trimming, micropolygon.cpp:754-835;
the per-hit test, micropolygon.cpp:1592-1627; CqTrimLoop / CqTrimLoopArray,
trimcurve.cpp:145-253): a plane over the unit (u, v) square trimmed by one
square loop keeps what lies inside the loop; two nested loops make a hole;
"outside" drops the fully trimmed micropolygons only."""
import numpy as np
import pytest

from aqsis_gb300 import scene as S
from tests import scenes_small as SS

N = 16  # pixels and micropolygons per side


def trimmed_plane(loops, outside=False, seed=4):
    fr = S.Frame(width=N, height=N, xsamples=2, ysamples=2, filter="box", xfilter=1.0, yfilter=1.0, q_dither=0.0)
    g = SS.plane(0, 0, N, N, 2.0, ci=np.ones(((N + 1) ** 2, 3)))
    u, v = np.meshgrid(np.arange(N + 1) / N, np.arange(N + 1) / N)
    g.trim_uv = np.stack([u.ravel(), v.ravel()], -1).astype(np.float32)
    g.trim_points = np.concatenate(loops).astype(np.float32) if loops else np.zeros((0, 2), np.float32)
    g.trim_loop_first = np.cumsum([0] + [len(l) for l in loops]).astype(np.int32)
    g.trim_set_first = np.array([0, len(loops)], np.int32)
    g.trim_set = np.array([0], np.int32)
    if outside:
        g.flags = g.flags | S.GRID_TRIM_OUTSIDE
    return SS.custom(fr, g, seed=seed, explicit=True)


def square(a, b):
    return np.array([[a, a], [b, a], [b, b], [a, b]], np.float32)


def sample_uv(sc):
    """(u, v) of every sample: raster position / N on this plane."""
    x0, y0, w, h = sc.frame.sample_region
    pos = np.asarray(sc.samples.pos, np.float32).reshape(-1, sc.frame.spp, 2)
    idx = np.asarray(sc.samples.pos_index).reshape(h, w) if sc.samples.pos_index is not None else \
        np.arange(h * w).reshape(h, w)
    px, py = np.meshgrid(np.arange(x0, x0 + w), np.arange(y0, y0 + h))
    p = pos[idx]  # (h, w, spp, 2)
    return ((px[..., None] + p[..., 0]) / N).ravel(), ((py[..., None] + p[..., 1]) / N).ravel()


def test_square_loop_keeps_its_inside(oracle):
    sc = trimmed_plane([square(0.25, 0.75)])
    hit = oracle.render(sc)["winner"] >= 0
    u, v = sample_uv(sc)
    far = (np.minimum(np.abs(u - 0.25), np.abs(u - 0.75)) > 0.02) | (np.minimum(np.abs(v - 0.25), np.abs(v - 0.75)) > 0.02)
    inside = (u > 0.25) & (u < 0.75) & (v > 0.25) & (v < 0.75)
    m = far & (u > 0) & (u < 1) & (v > 0) & (v < 1)
    assert np.array_equal(hit[m], inside[m])


def test_nested_loops_make_a_hole(oracle):
    sc = trimmed_plane([square(0.1, 0.9), square(0.4, 0.6)])
    hit = oracle.render(sc)["winner"] >= 0
    u, v = sample_uv(sc)
    ring = (u > 0.12) & (u < 0.88) & (v > 0.12) & (v < 0.88) & ~((u > 0.38) & (u < 0.62) & (v > 0.38) & (v < 0.62))
    hole = (u > 0.42) & (u < 0.58) & (v > 0.42) & (v < 0.58)
    assert hit[ring].all() and not hit[hole].any()


def test_no_loops_trims_nothing_inside_and_everything_outside(oracle):
    sc = trimmed_plane([])
    res = oracle.render(sc)
    u, v = sample_uv(sc)
    m = (u > 0.01) & (u < 0.99) & (v > 0.01) & (v < 0.99)
    assert (res["winner"][m] >= 0).all()
    # "outside" with no loops: every corner counts as trimmed and no edge
    # crosses a loop, so Split drops every micropolygon
    res = oracle.render(trimmed_plane([], outside=True))
    assert (res["winner"] < 0).all()


def test_outside_sense_has_no_test_at_the_hit(oracle):
    """With "outside" the per-hit test never rejects, so only micropolygons
    lying wholly inside the loop are dropped."""
    sc = trimmed_plane([square(0.25, 0.75)], outside=True)
    hit = oracle.render(sc)["winner"] >= 0
    u, v = sample_uv(sc)
    deep = (u > 0.32) & (u < 0.68) & (v > 0.32) & (v < 0.68)
    out = ((u < 0.2) | (u > 0.8) | (v < 0.2) | (v > 0.8)) & (u > 0.01) & (u < 0.99) & (v > 0.01) & (v < 0.99)
    assert not hit[deep].any() and hit[out].all()


def test_random_trims_run(oracle):
    base = SS.opaque_small(seed=41, scale=0.02)
    sc = S.with_trim(base, seed=2)
    a = oracle.render(base)["winner"] >= 0
    b = oracle.render(sc)["winner"] >= 0
    assert b.sum() < a.sum()


def test_scene_file_keeps_trims(tmp_path):
    sc = S.with_trim(SS.opaque_small(seed=42, scale=0.01), seed=3)
    p = tmp_path / "trim.npz"
    S.save_scene(str(p), sc)
    sc2, _ = S.load_scene(str(p))
    for k in ("trim_set", "trim_uv", "trim_points", "trim_loop_first", "trim_set_first", "flags"):
        assert np.array_equal(getattr(sc2.grids, k), getattr(sc.grids, k))
