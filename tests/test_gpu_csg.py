"""CSG on the device against the oracle: the two-solid known answers, random
trees over the small scenes (plain and batched), the host checks of
aqh_set_csg and the fragment limit of the device resolve."""
import numpy as np
import pytest

from aqsis_gb300 import scene as S
from tests import scenes_small as SS
from tests.test_csg import A_FACES, B_FACES, BLUE, RED, solids_scene
from tests.test_gpu_parity import compare

pytestmark = pytest.mark.gpu

KATS = {
    "union": lambda: solids_scene([S.CSG_UNION, 0, 0], [-1, 0, 0], A_FACES + B_FACES, [1, 1, 2, 2]),
    "intersection": lambda: solids_scene([S.CSG_INTERSECTION, 0, 0], [-1, 0, 0], A_FACES + B_FACES, [1, 1, 2, 2]),
    "difference": lambda: solids_scene([S.CSG_DIFFERENCE, 0, 0], [-1, 0, 0], A_FACES + B_FACES, [1, 1, 2, 2]),
    "difference_ba": lambda: solids_scene([S.CSG_DIFFERENCE, 0, 0], [-1, 0, 0], A_FACES + B_FACES, [2, 2, 1, 1]),
    "disjoint": lambda: solids_scene([S.CSG_INTERSECTION, 0, 0], [-1, 0, 0],
                                     [(2.0, RED), (3.0, RED), (4.0, BLUE), (5.0, BLUE)], [1, 1, 2, 2]),
    "nested": lambda: solids_scene([S.CSG_UNION, S.CSG_INTERSECTION, 0, 0, 0], [-1, 0, 1, 1, 0],
                                   A_FACES + B_FACES + [(6.0, BLUE), (7.0, BLUE)], [2, 2, 3, 3, 4, 4]),
    "two_trees": lambda: solids_scene([S.CSG_INTERSECTION, 0, 0, S.CSG_DIFFERENCE, 0, 0], [-1, 0, 0, -1, 3, 3],
                                      A_FACES + B_FACES + [(2.5, BLUE), (6.0, BLUE), (1.0, RED), (7.0, RED)],
                                      [1, 1, 2, 2, 4, 4, 5, 5]),
    "primitive_top": lambda: solids_scene([0], [-1], A_FACES + [(1.0, BLUE)], [0, 0, -1]),
}

RANDOM = {
    "opaque": lambda: S.with_csg(SS.opaque_small(seed=81, scale=0.02), seed=1),
    "transparent": lambda: S.with_csg(SS.transparent_small(seed=82, scale=0.03), seed=2),
    "motion_dof": lambda: S.with_csg(SS.motion_dof_small(seed=83, xs=4, ys=4, scale=0.02), seed=3),
    "motion_transparent": lambda: S.with_csg(SS.motion_dof_small(seed=84, xs=3, ys=3, scale=0.02,
                                                                 transparent=True), seed=4),
    "triangular": lambda: S.with_csg(SS.triangular_small(seed=85), seed=5),
    "edge_cases": lambda: S.with_csg(SS.edge_cases(seed=86), seed=6),
    "three_trees": lambda: S.with_csg(SS.transparent_small(seed=88, scale=0.02), seed=7, ntrees=3, frac=0.9),
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
def test_random_trees_match_oracle(aqh_lib, oracle, name, batched):
    sc = RANDOM[name]()
    compare(render(aqh_lib, sc, batched), oracle.render(sc))


def test_trees_are_checked(aqh_lib):
    from aqsis_gb300.aqh import AqhError
    sc = KATS["union"]()
    h = aqh_lib.Hider(0)
    try:
        h.frame_begin(sc.frame)
        bad = [
            ([5, 0, 0], [-1, 0, 0], [1, 2]),      # unknown node type
            ([1, 0, 0], [-1, 3, 0], [1, 2]),      # parent out of range
            ([1, 0, 0], [-1, 2, 0], [1, 2]),      # a primitive as parent
            ([1, 1, 0], [1, 0, 0], [2]),          # a cycle
            ([1, 0, 0], [-1, 0, 0], [1, 3]),      # grid node out of range
            ([1] + [0] * 33, [-1] + [0] * 33, [1]),  # 33 children
        ]
        for t, p, gn in bad:
            with pytest.raises(AqhError):
                h.set_csg(t, p, gn)
        h.set_csg([1, 0, 0], [-1, 0, 0], [1, 1, 2, 2])
        h.set_csg([], [], [])
    finally:
        h.close()


def test_fragment_limit_is_an_error(aqh_lib):
    """More than 24 hits at a sample with a CSG hit among them fails the
    render (the device resolve holds the sorted list in registers)."""
    from aqsis_gb300.aqh import AqhError
    faces = [(2.0 + 0.25 * k, RED if k % 2 == 0 else BLUE) for k in range(26)]
    sc = solids_scene([S.CSG_UNION] + [0] * 13, [-1] + [0] * 13, faces, [1 + k // 2 for k in range(26)])
    h = aqh_lib.Hider(0)
    try:
        with pytest.raises(AqhError):
            h.render_scene(sc)
        # the context stays usable
        ok = KATS["union"]()
        h.render_scene(ok)
    finally:
        h.close()
