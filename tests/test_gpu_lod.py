"""Level-of-detail bounds on the device against the oracle."""
import pytest

from aqsis_gb300 import scene as S
from tests import scenes_small as SS
from tests.test_gpu_parity import compare

pytestmark = pytest.mark.gpu

SCENES = {
    "opaque": lambda: S.with_lod(SS.opaque_small(seed=71, scale=0.03), seed=1),
    "transparent": lambda: S.with_lod(SS.transparent_small(seed=72, scale=0.03), seed=2),
    "edge_cases": lambda: S.with_lod(SS.edge_cases(seed=73), seed=3),
    "motion_dof": lambda: S.with_lod(SS.motion_dof_small(seed=74, xs=4, ys=4, scale=0.02), seed=4),
    "motion_transparent": lambda: S.with_lod(SS.motion_dof_small(seed=75, xs=3, ys=3, scale=0.02,
                                                                 transparent=True), seed=5),
}


@pytest.mark.parametrize("batched", [False, True])
@pytest.mark.parametrize("name", sorted(SCENES))
def test_detail_bounds_match_oracle(aqh_lib, oracle, name, batched):
    sc = SCENES[name]()
    h = aqh_lib.Hider(0)
    try:
        h.set_mode(batched)
        res = h.render_scene(sc)
    finally:
        h.close()
    compare(res, oracle.render(sc))
