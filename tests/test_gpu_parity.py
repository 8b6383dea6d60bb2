"""GPU hider vs the CPU oracle on the same seeded inputs.

Bit-exact: per-sample winning micropolygon ids (the occluding hit before
Combine), occlZ, transparent fragment counts and valid masks.  Composited
samples and filtered pixels: within 1e-5 relative (absolute 1e-6 near zero);
8-bit quantized values: within 1 LSB.  In practice both are exact because
the device follows the reference's operation order without FMA contraction.
"""
import numpy as np
import pytest

from tests import scenes_small as SS

pytestmark = pytest.mark.gpu

REL = 1e-5
ABS = 1e-6


def close_or_same(a, b):
    """Within REL/ABS, or the same non-finite value (the reference's own z
    channel overflows to inf/NaN where FLT_MAX depths meet negative filter
    lobes)."""
    with np.errstate(invalid="ignore", over="ignore"):
        d = np.abs(a - b)
        ok = (d <= REL * np.abs(b)) | (d <= ABS)
    ok |= (np.isnan(a) & np.isnan(b)) | (np.isinf(a) & (a == b))
    return ok


def compare(res, ref, exact_pixels=False):
    assert np.array_equal(res["winner"], ref["winner"]), \
        "winner mismatch at %d samples" % int((res["winner"] != ref["winner"]).sum())
    assert np.array_equal(res["occlz"].view(np.uint32), ref["occlz"].view(np.uint32))
    assert np.array_equal(res["nfrag"], ref["nfrag"])
    assert np.array_equal(res["valid"], ref["valid"])
    ok = close_or_same(res["sdata"], ref["sdata"])
    assert ok.all(), "sample data differs at %d entries" % int((~ok).sum())
    ca, cb = res["channels"], ref["channels"]
    ok = close_or_same(ca, cb)
    assert ok.all(), "channels differ at %d entries" % int((~ok).sum())
    q = np.abs(res["quantized"].astype(np.int32) - ref["quantized"].astype(np.int32))
    assert q.max() <= 1
    if exact_pixels:
        assert np.array_equal(ca.view(np.uint32), cb.view(np.uint32))
        assert q.max() == 0


def run_both(hider, oracle, scene, qch=(0, 1, 2, 6)):
    res = hider.render_scene(scene, qch)
    ref = oracle.render(scene, qch)
    return res, ref


def test_opaque_stream_small(hider, oracle):
    res, ref = run_both(hider, oracle, SS.opaque_small(seed=11))
    compare(res, ref, exact_pixels=True)
    assert res["valid"].mean() > 0.5


def test_opaque_stream_explicit_samples(hider, oracle):
    res, ref = run_both(hider, oracle, SS.opaque_small(seed=12, explicit=True))
    compare(res, ref, exact_pixels=True)


@pytest.mark.parametrize("xs,ys", [(1, 1), (2, 2), (3, 3), (4, 4), (5, 3), (8, 8)])
def test_edge_cases_sample_counts(hider, oracle, xs, ys):
    res, ref = run_both(hider, oracle, SS.edge_cases(seed=20 + xs, xs=xs, ys=ys))
    compare(res, ref, exact_pixels=True)


@pytest.mark.parametrize("filt", [("box", 1.0, 1.0), ("catmull-rom", 3.0, 3.0), ("sinc", 4.0, 4.0),
                                  ("triangle", 2.5, 1.5), ("mitchell", 4.0, 4.0), ("disk", 3.0, 3.0)])
def test_edge_cases_filters(hider, oracle, filt):
    res, ref = run_both(hider, oracle, SS.edge_cases(seed=31, filt=filt))
    compare(res, ref, exact_pixels=True)


def test_transparent_small(hider, oracle):
    res, ref = run_both(hider, oracle, SS.transparent_small(seed=41))
    compare(res, ref)
    assert res["nfrag"].max() > 1


@pytest.mark.parametrize("xs,ys", [(3, 3), (8, 8)])
def test_transparent_edge_cases(hider, oracle, xs, ys):
    res, ref = run_both(hider, oracle, SS.transparent_edge(seed=42, xs=xs, ys=ys))
    compare(res, ref)


def test_transparent_frame_with_unflagged_occluder(hider, oracle):
    res, ref = run_both(hider, oracle, SS.transparent_hidden_occluder())
    compare(res, ref)
    assert (res["winner"] >= 0).any()  # the unflagged grid does occlude


@pytest.mark.parametrize("scene_fn", [lambda: SS.triangular_small(),
                                      lambda: SS.triangular_motion_small(dof=False),
                                      lambda: SS.triangular_motion_small(dof=True),
                                      lambda: SS.triangular_transparent_small()],
                         ids=["static", "motion", "motion_dof", "transparent"])
def test_triangular_grids(hider, oracle, scene_fn):
    sc = scene_fn()
    res, ref = run_both(hider, oracle, sc)
    compare(res, ref)


def test_crop_window_and_exposure(hider, oracle):
    sc = SS.edge_cases(seed=51)
    sc.frame.crop = (7, 50, 5, 40)
    sc.frame.gain, sc.frame.gamma = 1.7, 2.2
    from aqsis_gb300 import scene as S
    sc.samples = S.make_samples(sc.frame, np.random.default_rng(3), 32, dither=True)
    sc.frame.q_dither = 0.5
    res, ref = run_both(hider, oracle, sc)
    compare(res, ref)


def test_quantized_channel_orders(hider, oracle):
    sc = SS.edge_cases(seed=61)
    for qch in [(6, 0, 1, 2), (0, 1, 2), (7,), (8, 6)]:
        res, ref = run_both(hider, oracle, sc, qch)
        q = np.abs(res["quantized"].astype(np.int32) - ref["quantized"].astype(np.int32))
        assert q.max() <= 1, qch


def test_empty_frame(hider, oracle):
    from aqsis_gb300 import scene as S
    fr = S.Frame(width=33, height=17, xsamples=2, ysamples=2, q_dither=0.0)
    g = SS.plane(200, 200, 2, 2, 5.0)  # entirely outside
    sc = SS.custom(fr, g)
    res, ref = run_both(hider, oracle, sc)
    compare(res, ref, exact_pixels=True)
    assert not res["valid"].any()


def test_bucket_readback_matches_channels(hider, oracle):
    sc = SS.edge_cases(seed=71)
    res = hider.render_scene(sc)
    ch = res["channels"]
    b = hider.read_bucket(1, 2)
    assert np.array_equal(b, ch[32:48, 16:32])
    b = hider.read_bucket(3, 2)  # partial bucket at the right edge (64 = 4*16, so full)
    assert b.shape[1] == 16


def test_device_invbilinear_matches_oracle(aqh_lib, oracle):
    from tests.test_oracle_bilinear import CASES, fixture_uv, quad_array
    for name, quad, ex, rel, ab in CASES:
        q = quad_array(quad)
        P = oracle.bilerp2(q, fixture_uv(*ex))
        a = aqh_lib.invbilinear(q, P)
        b = oracle.invbilinear(q, P)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), name


def test_motion_blur_and_dof(hider, oracle):
    res, ref = run_both(hider, oracle, SS.motion_dof_small(seed=81))
    compare(res, ref, exact_pixels=True)


def test_motion_blur_only(hider, oracle):
    res, ref = run_both(hider, oracle, SS.motion_dof_small(seed=82, dof=False, xs=4, ys=4))
    compare(res, ref, exact_pixels=True)


def test_dof_only(hider, oracle):
    res, ref = run_both(hider, oracle, SS.dof_only_small(seed=83))
    compare(res, ref, exact_pixels=True)


@pytest.mark.parametrize("dof", [False, True], ids=["motion", "motion_dof"])
def test_motion_blur_with_static_grids(hider, oracle, dof):
    res, ref = run_both(hider, oracle, SS.motion_mixed_small(seed=85, dof=dof))
    compare(res, ref, exact_pixels=True)


def test_motion_blur_transparent(hider, oracle):
    res, ref = run_both(hider, oracle, SS.motion_dof_small(seed=84, dof=False, xs=3, ys=3, transparent=True))
    compare(res, ref)


@pytest.mark.parametrize("scene_fn", [lambda: SS.opaque_small(seed=101), lambda: SS.transparent_small(seed=102),
                                      lambda: SS.edge_cases(seed=103), lambda: SS.motion_dof_small(seed=104)],
                         ids=["opaque", "transparent", "edge", "mbdof"])
def test_batched_mode_matches_oracle_and_replays(hider, oracle, scene_fn):
    """AQH_MODE_BATCHED (persistent tile queue, CUDA graph) gives the oracle's
    pixels, and replaying the captured graph gives the same bits again."""
    sc = scene_fn()
    ref = oracle.render(sc)
    hider.set_mode(True)
    try:
        res = hider.render_scene(sc)
        compare(res, ref)
        again = []
        for _ in range(2):
            hider.render(sync=True)
            again.append(hider.read_channels())
        for a in again:
            assert np.array_equal(a.view(np.uint32), res["channels"].view(np.uint32))
    finally:
        hider.set_mode(False)


@pytest.mark.parametrize("transparent", [False, True])
def test_static_grid_behind_eye_in_motion_frame(hider, oracle, transparent):
    """RenderMPG_MBOrDof's clipping-range cull applies to moving micropolygons
    only; a static grid at negative depth in a motion-blurred frame is still
    sampled (found by the random differential frames)."""
    sc = SS.motion_static_behind_eye(transparent=transparent)
    res, ref = run_both(hider, oracle, sc)
    compare(res, ref)
    assert (ref["winner"] >= 0).sum() + (ref["nfrag"] > 0).sum() > 0


@pytest.mark.parametrize("xs,ys", [(5, 5), (6, 6), (8, 8)])
@pytest.mark.parametrize("filt", [("gaussian", 2.0, 2.0), ("catmull-rom", 3.0, 3.0)], ids=["gaussian", "catmull-rom"])
def test_rolling_filter_windows(hider, oracle, xs, ys, filt):
    """3x3 windows above 16 samples per pixel take the rolling-window filter:
    crop windows whose height is not a multiple of its 8-row runs, exposure
    gain (bit-exact); with a gamma the device's pow may differ from the
    reference's float pow by an ulp, so that case is held to the tolerance."""
    sc = SS.edge_cases(seed=81 + xs, xs=xs, ys=ys, filt=filt)
    sc.frame.crop = (3, sc.frame.width - 4, 2, sc.frame.height - 5)
    sc.frame.gain = 1.3
    res, ref = run_both(hider, oracle, sc)
    compare(res, ref, exact_pixels=True)
    sc.frame.gamma = 1.8
    res, ref = run_both(hider, oracle, sc)
    compare(res, ref)


@pytest.mark.parametrize("offsets", ["outside", "edges"])
def test_rolling_filter_offsets(hider, oracle, offsets):
    """The rolling-window filter skips the window test only when every sample
    offset lies in [0, 1] (a 3x3 neighbourhood then lies inside every window
    of half-width 1.5).  Offsets reaching outside the pixel take the test
    (`outside`); offsets of exactly 0 and 1 put samples on the window's
    inclusive edges, -1.5 and +1.5 from the centre (`edges`)."""
    sc = SS.edge_cases(seed=95, xs=6, ys=6, filt=("catmull-rom", 3.0, 3.0))
    pos = np.array(sc.samples.pos, dtype=np.float32, copy=True)
    if offsets == "outside":
        pos = pos * np.float32(1.3) - np.float32(0.15)
    else:
        flat = pos.reshape(-1, 2)
        flat[0::3] = 0.0
        flat[1::3] = 1.0
    sc.samples.pos = pos
    res, ref = run_both(hider, oracle, sc)
    compare(res, ref, exact_pixels=True)
