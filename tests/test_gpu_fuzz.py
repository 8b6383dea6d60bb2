"""Differential tests on random small frames (tests/scenes_small.fuzz): the
device hider against the oracle at the parity bars, in both execution forms."""
import pytest

from tests import scenes_small as SS
from tests.test_gpu_parity import compare

pytestmark = pytest.mark.gpu

SEEDS = list(range(300))


@pytest.mark.parametrize("seed", SEEDS)
def test_random_frame_matches_oracle(hider, oracle, seed):
    sc = SS.fuzz(seed)
    compare(hider.render_scene(sc), oracle.render(sc))


@pytest.mark.parametrize("seed", SEEDS[:100])
def test_random_frame_batched(aqh_lib, oracle, seed):
    sc = SS.fuzz(seed)
    h = aqh_lib.Hider(0)
    try:
        h.set_mode(True)
        res = h.render_scene(sc)
    finally:
        h.close()
    compare(res, oracle.render(sc))


@pytest.mark.parametrize("seed", SEEDS[:150])
def test_random_frame_with_solids(aqh_lib, oracle, seed):
    """Random frames with random CSG trees over their grids.  The device
    refuses (AQH_ELIMIT) a sample holding a CSG hit among more than 24 hits
    or a NaN depth; the oracle's hit counts must then show such a sample."""
    import numpy as np
    from aqsis_gb300 import scene as S
    from aqsis_gb300.aqh import AqhError
    sc = S.with_csg(SS.fuzz(seed), seed=seed, ntrees=1 + seed % 3)
    ref = oracle.render(sc)
    h = aqh_lib.Hider(0)
    try:
        h.set_mode(seed % 2 == 1)
        try:
            res = h.render_scene(sc)
        except AqhError:
            ntot = ref["nfrag"] + (ref["winner"] >= 0)
            assert ntot.max() > 24 or np.isnan(ref["occlz"]).any() or np.isnan(sc.grids.P).any()
            return
    finally:
        h.close()
    compare(res, ref)


@pytest.mark.parametrize("seed", SEEDS[:150])
def test_random_frame_with_trims(aqh_lib, oracle, seed):
    """Random frames with random trim sets over their grids."""
    from aqsis_gb300 import scene as S
    sc = S.with_trim(SS.fuzz(seed), seed=seed, frac=0.4 + 0.6 * (seed % 5) / 4)
    h = aqh_lib.Hider(0)
    try:
        h.set_mode(seed % 2 == 1)
        res = h.render_scene(sc)
    finally:
        h.close()
    compare(res, oracle.render(sc))


def _positive_depth_seeds(n):
    """Random frames whose depths are all positive (camera space needs them)."""
    import numpy as np
    out = []
    for s in range(1000):
        if len(out) == n:
            break
        if not (np.asarray(SS.fuzz(s).grids.P)[:, 2] <= 0).any():
            out.append(s)
    return out


@pytest.mark.parametrize("seed", _positive_depth_seeds(60))
def test_random_frame_with_culling(aqh_lib, oracle, seed):
    """Random frames turned to camera space (every other grid) with random
    normals and trailing black opacity culled on the device."""
    from aqsis_gb300 import scene as S
    sc = S.with_culling(S.to_camera_space(SS.fuzz(seed), every=2), seed=seed)
    h = aqh_lib.Hider(0)
    try:
        h.set_mode(seed % 2 == 1)
        res = h.render_scene(sc)
    finally:
        h.close()
    compare(res, oracle.render(sc), exact_pixels=False)
