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
