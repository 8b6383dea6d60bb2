"""Split's projection on the device (AQH_GRID_CAMERA + aqh_set_camera_to_raster)
against the oracle's projection followed by the oracle hider, through each
way of submitting grids: per-grid host submits, packed host arrays and
device-resident arrays (projected in place, flag cleared)."""
import numpy as np
import pytest

from aqsis_gb300 import scene as S
from tests import scenes_small as SS
from tests.test_gpu_parity import compare

pytestmark = pytest.mark.gpu


def _finish(hider, qch=(0, 1, 2, 6)):
    hider.render(sync=True)
    res = {"channels": hider.read_channels(), "quantized": hider.read_quantized(qch)}
    res.update(hider.read_samples())
    return res


def render_packed(hider, sc):
    hider.frame_begin(sc.frame)
    hider.set_samples(sc.samples)
    hider.submit_grids_host(sc.grids)
    return _finish(hider)


def render_device(hider, sc, times=1):
    torch = pytest.importorskip("torch")
    g = sc.grids
    dev = torch.device("cuda", 0)
    dtypes = {"cu": np.int32, "cv": np.int32, "nkeys": np.int32, "flags": np.int32, "pbase": np.int64,
              "cbase": np.int64, "tbase": np.int32, "times": np.float32, "P": np.float32, "Ci": np.float32,
              "Oi": np.float32}
    t = {k: torch.from_numpy(np.ascontiguousarray(getattr(g, k), dt)).to(dev) for k, dt in dtypes.items()}
    torch.cuda.synchronize()  # the hider's own stream does not wait for torch's
    out = []
    hider.frame_begin(sc.frame)
    hider.set_samples(sc.samples)
    hider.submit_grids_device(g.ngrids, t["cu"].data_ptr(), t["cv"].data_ptr(), t["nkeys"].data_ptr(),
                              t["flags"].data_ptr(), t["pbase"].data_ptr(), t["cbase"].data_ptr(),
                              t["tbase"].data_ptr(), t["times"].data_ptr(), t["P"].data_ptr(), t["Ci"].data_ptr(),
                              t["Oi"].data_ptr(), g.micropolygons)
    for _ in range(times):
        out.append(_finish(hider))
    torch.cuda.synchronize()
    return out, {k: v.cpu().numpy() for k, v in t.items()}


SCENES = {
    "perspective_static": lambda: SS.camera_small(seed=31),
    "orthographic_static": lambda: SS.camera_small(seed=32, every=1, orthographic=True),
    "perspective_triangular": lambda: S.to_camera_space(SS.triangular_small(seed=33), every=2),
    "perspective_motion_dof": lambda: S.to_camera_space(SS.triangular_motion_small(seed=34)),
    "perspective_transparent": lambda: S.to_camera_space(SS.transparent_small(seed=35, scale=0.03), every=2),
    "spheres": lambda: __import__("aqsis_gb300.spheres", fromlist=["x"]).sphere_scene(seed=3, nspheres=12,
                                                                                      width=160, height=120),
}


@pytest.mark.parametrize("name", sorted(SCENES))
def test_camera_grids_match_oracle(hider, oracle, name):
    sc = SCENES[name]()
    assert (sc.grids.flags & S.GRID_CAMERA).any()
    res = hider.render_scene(sc)
    ref = oracle.render(sc)
    # transparent frames: the z channel's NaNs (FLT_MAX depths under negative
    # filter lobes) may carry another payload, so compare values, not bits
    compare(res, ref, exact_pixels="transparent" not in name)


def test_camera_grids_packed_host(hider, oracle):
    sc = SS.camera_small(seed=36)
    res = render_packed(hider, sc)
    compare(res, oracle.render(sc), exact_pixels=True)
    # the packed arrays are uploaded again for every render: same frame
    hider.render(sync=True)
    compare(_finish(hider), oracle.render(sc), exact_pixels=True)


def test_camera_grids_device_in_place(hider, oracle):
    sc = S.to_camera_space(SS.motion_mixed_small(seed=37), every=2)
    outs, after = render_device(hider, sc, times=2)
    ref = oracle.render(sc)
    for res in outs:
        compare(res, ref, exact_pixels=True)
    # Split leaves the device arrays in hybrid raster space with the flag cleared
    proj = oracle.projected_grids(sc)
    assert not (after["flags"] & S.GRID_CAMERA).any()
    assert np.array_equal(after["P"].view(np.uint32), proj.P.view(np.uint32))


def test_camera_flag_without_matrix_is_rejected(hider):
    from aqsis_gb300.aqh import AqhError
    import dataclasses
    sc = SS.camera_small(seed=38)
    sc = S.Scene(dataclasses.replace(sc.frame, camera_to_raster=None), sc.grids, sc.samples)
    with pytest.raises(AqhError):
        hider.render_scene(sc)


@pytest.mark.parametrize("name", ["perspective_static", "perspective_motion_dof", "perspective_transparent"])
def test_three_float_host_grids(aqh_lib, oracle, name):
    """aqh_submit_grids_host3 (CqVector3D / CqColor layout, widened on the
    device) renders exactly what the float4 arrays render."""
    sc = SCENES[name]()
    ref = oracle.render(sc)
    h = aqh_lib.Hider(0)
    try:
        for batched, engines in ((False, False), (True, False), (True, True)):
            h.set_mode(batched)
            h.set_host_copy(engines)
            h.frame_begin(sc.frame)
            h.set_samples(sc.samples)
            h.submit_grids_host(sc.grids, packed3=True)
            compare(_finish(h), ref, exact_pixels="transparent" not in name)
    finally:
        h.close()
