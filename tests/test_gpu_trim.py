"""Trim curves on the device against the oracle: the known-answer planes,
random trim sets over the small scenes (static, depth of field and motion
blur, plain and batched), and the host and device checks of aqh_set_trim."""
import numpy as np
import pytest

from aqsis_gb300 import scene as S
from tests import scenes_small as SS
from tests.test_gpu_parity import compare
from tests.test_trim import square, trimmed_plane

pytestmark = pytest.mark.gpu

KATS = {
    "square": lambda: trimmed_plane([square(0.25, 0.75)]),
    "hole": lambda: trimmed_plane([square(0.1, 0.9), square(0.4, 0.6)]),
    "no_loops": lambda: trimmed_plane([]),
    "no_loops_outside": lambda: trimmed_plane([], outside=True),
    "outside": lambda: trimmed_plane([square(0.25, 0.75)], outside=True),
}

RANDOM = {
    "opaque": lambda: S.with_trim(SS.opaque_small(seed=91, scale=0.02), seed=1),
    "transparent": lambda: S.with_trim(SS.transparent_small(seed=92, scale=0.03), seed=2),
    "dof": lambda: S.with_trim(SS.dof_only_small(seed=93, scale=0.02), seed=3),
    "motion_dof": lambda: S.with_trim(SS.motion_dof_small(seed=94, xs=4, ys=4, scale=0.02), seed=4),
    "motion_mixed": lambda: S.with_trim(SS.motion_mixed_small(seed=95, scale=0.02), seed=5),
    "motion_transparent": lambda: S.with_trim(SS.motion_dof_small(seed=96, xs=3, ys=3, scale=0.02,
                                                                  transparent=True), seed=6),
    "triangular": lambda: S.with_trim(SS.triangular_small(seed=97), seed=7),
    "edge_cases": lambda: S.with_trim(SS.edge_cases(seed=98), seed=8),
    "with_csg": lambda: S.with_csg(S.with_trim(SS.transparent_small(seed=99, scale=0.02), seed=9), seed=9),
}


def render(aqh_lib, sc, batched=False):
    h = aqh_lib.Hider(0)
    try:
        h.set_mode(batched)
        return h.render_scene(sc)
    finally:
        h.close()


@pytest.mark.parametrize("name", sorted(KATS))
def test_known_answers_match_oracle(aqh_lib, oracle, name):
    sc = KATS[name]()
    compare(render(aqh_lib, sc), oracle.render(sc))


@pytest.mark.parametrize("batched", [False, True])
@pytest.mark.parametrize("name", sorted(RANDOM))
def test_random_trims_match_oracle(aqh_lib, oracle, name, batched):
    sc = RANDOM[name]()
    compare(render(aqh_lib, sc, batched), oracle.render(sc))


def test_trim_sets_are_checked(aqh_lib):
    from aqsis_gb300.aqh import AqhError
    sc = KATS["square"]()
    g = sc.grids
    h = aqh_lib.Hider(0)
    try:
        h.frame_begin(sc.frame)
        pts, lf, sf = g.trim_points, g.trim_loop_first, g.trim_set_first
        bad = [
            ([1], pts, lf, sf),                                   # set out of range
            ([0], pts, np.array([0, 9], np.int32), sf),           # loop past the points
            ([0], pts, np.array([2, 1, 4], np.int32), np.array([0, 2], np.int32)),  # decreasing loop starts
            ([0], pts, lf, np.array([0, 2], np.int32)),           # set past the loops
        ]
        for gs, p, l, s in bad:
            with pytest.raises(AqhError):
                h.set_trim(gs, g.trim_uv, p, l, s)
        h.set_trim([0], g.trim_uv, pts, lf, sf)
        h.set_trim([], np.zeros((0, 2)), np.zeros((0, 2)), [0], [0])
    finally:
        h.close()


def test_short_uv_array_is_an_error(aqh_lib):
    """A trimmable grid whose vertices run past the uv array is refused by
    the device check before any sampling; the context stays usable."""
    from aqsis_gb300.aqh import AqhError
    sc = KATS["square"]()
    sc.grids.trim_uv = sc.grids.trim_uv[:10]
    h = aqh_lib.Hider(0)
    try:
        with pytest.raises(AqhError):
            h.render_scene(sc)
        h.render_scene(KATS["hole"]())
    finally:
        h.close()
