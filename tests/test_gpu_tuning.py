"""Launch-shape tuning (aqh_set_tuning / aqh_autotune): any tile size,
super-tile size or persistent CTA count gives bit-identical results, and the
autotuner leaves a valid choice set on the context."""
import numpy as np
import pytest

from tests import scenes_small as SS

pytestmark = pytest.mark.gpu

KEYS = ("winner", "occlz", "nfrag", "valid", "sdata", "channels", "quantized")

SCENES = {
    "opaque": lambda: SS.opaque_small(seed=21),
    "transparent": lambda: SS.transparent_small(seed=22),
    "hidden_occluder": lambda: SS.transparent_hidden_occluder(seed=23),
    "motion_mixed": lambda: SS.motion_mixed_small(seed=24),
    "motion_dof": lambda: SS.motion_dof_small(seed=25),
    "triangular": lambda: SS.triangular_small(seed=26),
}

TUNINGS = [
    (0, 0, 0, 1),   # one filter tile in flight per SM
    (0, 0, 0, 8),
    (0, 64, 0),
    (0, 256, 0),
    (64, 0, 0),
    (255, 0, 0),    # 15 x 17 pixels clamps to 15 x 16
    (16, 32, 0),
    (100, 1000, 0),
]


def same(a, b):
    for k in KEYS:
        x, y = np.asarray(a[k]), np.asarray(b[k])
        assert x.shape == y.shape, k
        assert np.array_equal(x.view(np.uint8), y.view(np.uint8)), "%s differs" % k


@pytest.fixture()
def own_hider(aqh_lib):
    h = aqh_lib.Hider(0)
    yield h
    h.close()


@pytest.mark.parametrize("name", sorted(SCENES))
def test_tilings_give_identical_results(own_hider, name):
    sc = SCENES[name]()
    base = own_hider.render_scene(sc)
    for t in TUNINGS:
        own_hider.set_tuning(*t)
        assert own_hider.get_tuning()["tile_pixels"] == t[0]
        res = own_hider.render_scene(sc)
        same(res, base)
    own_hider.set_tuning()


@pytest.mark.parametrize("name", ["opaque", "transparent", "motion_mixed"])
def test_batched_tilings_give_identical_results(own_hider, name):
    sc = SCENES[name]()
    base = own_hider.render_scene(sc)
    own_hider.set_mode(True)
    for t in [(0, 0, 3), (64, 64, 1), (16, 0, 0)]:
        own_hider.set_tuning(*t)
        res = own_hider.render_scene(sc)
        same(res, base)


@pytest.mark.parametrize("batched", [False, True])
def test_autotune_keeps_results(own_hider, batched):
    sc = SS.opaque_small(seed=27)
    base = own_hider.render_scene(sc)
    own_hider.set_mode(batched)
    own_hider.frame_begin(sc.frame)
    own_hider.set_samples(sc.samples)
    own_hider.submit_scene_grids(sc.grids)
    best = own_hider.autotune(repeats=2)
    assert best["ms"] > 0
    assert own_hider.get_tuning()["tile_pixels"] == best["tile_pixels"]
    assert own_hider.get_tuning()["supertile_pixels"] == best["supertile_pixels"]
    res = own_hider.render_scene(sc)
    same(res, base)


def test_tuning_rejects_out_of_range(own_hider):
    from aqsis_gb300.aqh import AqhError
    with pytest.raises(AqhError):
        own_hider.set_tuning(tile_pixels=-1)
    with pytest.raises(AqhError):
        own_hider.set_tuning(tile_pixels=257)
