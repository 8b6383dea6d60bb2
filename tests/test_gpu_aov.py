"""Output variables on the device (aqh_set_aov_count / aqh_read_aov) against
the oracle, through per-grid, packed-host and device-resident submission and
in the batched form."""
import numpy as np
import pytest

from aqsis_gb300 import scene as S
from tests import scenes_small as SS
from tests.test_gpu_parity import close_or_same, compare

pytestmark = pytest.mark.gpu

SCENES = {
    "opaque": lambda: S.with_aov(SS.opaque_small(seed=61, scale=0.03), 3, seed=1),
    "transparent": lambda: S.with_aov(SS.transparent_small(seed=62, scale=0.03), 2, seed=2),
    "edge_cases": lambda: S.with_aov(SS.edge_cases(seed=63), 1, seed=3),
    "motion_dof_transparent": lambda: S.with_aov(SS.motion_dof_small(seed=64, xs=3, ys=3, scale=0.02,
                                                                     transparent=True), 4, seed=4),
    "triangular": lambda: S.with_aov(SS.triangular_small(seed=65), 2, seed=5),
}


def check(res, ref):
    compare(res, ref)
    ok = close_or_same(res["aov"], ref["aov"])
    assert ok.all(), "output variables differ at %d entries" % int((~ok).sum())


@pytest.mark.parametrize("name", sorted(SCENES))
def test_output_variables_match_oracle(hider, oracle, name):
    sc = SCENES[name]()
    check(hider.render_scene(sc), oracle.render(sc))


def test_output_variables_packed_and_batched(aqh_lib, oracle):
    sc = SCENES["transparent"]()
    ref = oracle.render(sc)
    h = aqh_lib.Hider(0)
    try:
        for batched in (False, True):
            h.set_mode(batched)
            h.frame_begin(sc.frame)
            h.set_samples(sc.samples)
            h.submit_grids_host(sc.grids)
            h.render(sync=True)
            got = h.read_aov()
            assert np.array_equal(got.view(np.uint32), ref["aov"].view(np.uint32)) or close_or_same(got, ref["aov"]).all()
            # a display request can name output variable k as channel 9 + k
            d = h.read_display((9, 10), one=0.0, qmin=0.0, qmax=0.0, dither_amp=0.0)
            assert np.array_equal(d.view(np.uint32), got.view(np.uint32))
    finally:
        h.close()


def test_output_variables_device_grids(aqh_lib, oracle):
    torch = pytest.importorskip("torch")
    sc = SCENES["opaque"]()
    g = sc.grids
    dev = torch.device("cuda", 0)
    dtypes = {"cu": np.int32, "cv": np.int32, "nkeys": np.int32, "flags": np.int32, "pbase": np.int64,
              "cbase": np.int64, "tbase": np.int32, "times": np.float32, "P": np.float32, "Ci": np.float32,
              "Oi": np.float32, "aov": np.float32}
    t = {k: torch.from_numpy(np.ascontiguousarray(getattr(g, k), dt)).to(dev) for k, dt in dtypes.items()}
    torch.cuda.synchronize()
    h = aqh_lib.Hider(0)
    try:
        h.frame_begin(sc.frame)
        h.set_samples(sc.samples)
        h.set_aov_count(g.aov.shape[1])
        h.submit_grids_device(g.ngrids, *[t[k].data_ptr() for k in ("cu", "cv", "nkeys", "flags", "pbase", "cbase",
                                                                    "tbase", "times", "P", "Ci", "Oi")],
                              g.micropolygons)
        h._check(h.L.aqh_submit_aov_device(h.ctx, t["aov"].data_ptr()), "aqh_submit_aov_device")
        h.render(sync=True)
        got = h.read_aov()
    finally:
        h.close()
    ref = oracle.render(sc)
    assert np.array_equal(got.view(np.uint32), ref["aov"].view(np.uint32))
