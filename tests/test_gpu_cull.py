"""Shade / Split culling on the device against the oracle: random normals
and trailing black opacity over camera-space scenes (static, motion blur,
transparent), plain and batched, host and three-float host grids."""
import pytest

from aqsis_gb300 import scene as S
from tests import scenes_small as SS
from tests.test_gpu_parity import compare

pytestmark = pytest.mark.gpu

SCENES = {
    "static": lambda: S.with_culling(SS.camera_small(seed=63, every=1), seed=1),
    "mixed": lambda: S.with_culling(SS.camera_small(seed=64, every=2), seed=2),
    "motion": lambda: S.with_culling(S.to_camera_space(SS.motion_dof_small(seed=65, xs=4, ys=4, scale=0.02)),
                                     seed=3),
    "transparent": lambda: S.with_culling(S.to_camera_space(SS.transparent_small(seed=66, scale=0.02)), seed=4),
    "with_trims": lambda: S.with_trim(S.with_culling(SS.camera_small(seed=67, every=1), seed=5), seed=5),
}


@pytest.mark.parametrize("batched", [False, True])
@pytest.mark.parametrize("name", sorted(SCENES))
def test_culling_matches_oracle(aqh_lib, oracle, name, batched):
    sc = SCENES[name]()
    h = aqh_lib.Hider(0)
    try:
        h.set_mode(batched)
        res = h.render_scene(sc)
    finally:
        h.close()
    compare(res, oracle.render(sc), exact_pixels="transparent" not in name)


def test_culling_three_float_host_grids(aqh_lib, oracle):
    from tests.test_gpu_camera import _finish
    sc = SCENES["static"]()
    h = aqh_lib.Hider(0)
    try:
        h.frame_begin(sc.frame)
        h.set_samples(sc.samples)
        h.submit_grids_host(sc.grids, packed3=True)
        compare(_finish(h), oracle.render(sc))
    finally:
        h.close()


def test_short_normals_are_an_error(aqh_lib):
    from aqsis_gb300.aqh import AqhError
    sc = SCENES["static"]()
    sc.grids.cull_Ng = sc.grids.cull_Ng[:5]
    h = aqh_lib.Hider(0)
    try:
        with pytest.raises(AqhError):
            h.render_scene(sc)
    finally:
        h.close()
