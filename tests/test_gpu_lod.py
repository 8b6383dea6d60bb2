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


def test_sample_tables_are_checked(aqh_lib):
    """A table without pattern choices needs one pattern per pixel, and
    choices must name existing patterns: both are refused on the host
    before anything reads them."""
    import dataclasses
    import numpy as np
    from aqsis_gb300.aqh import AqhError
    sc = SS.opaque_small(seed=76, scale=0.02)
    smp = sc.samples
    assert smp.pos_index is not None and smp.npatterns < sc.frame.sample_region[2] * sc.frame.sample_region[3]
    n = np.asarray(smp.pos).reshape(-1, 2).shape[0]
    h = aqh_lib.Hider(0)
    try:
        h.frame_begin(sc.frame)
        with pytest.raises(AqhError):
            h.set_samples(dataclasses.replace(smp, lod=np.zeros(n, np.float32), lod_index=None))
        bad = np.array(smp.pos_index, np.uint32, copy=True)
        bad[3] = smp.npatterns
        with pytest.raises(AqhError):
            h.set_samples(dataclasses.replace(smp, pos_index=bad))
    finally:
        h.close()
