"""GPU hider vs the CPU oracle at the benchmarked sizes.

The small parity scenes (tests/test_gpu_parity.py) run at a few percent of
the benchmark frames.  These run the benchmark workloads themselves, or the
bounded slices of them that the CPU baseline renders, in both execution
forms (plain: one launch per stage; batched: the persistent tile queue and
the per-frame CUDA graph), so that the super-tile lists, the tile queue and
the sample store are checked at the sizes that are timed:

* the opaque 1080p stream's 768x432 slice (32,000 grids, 8.2M
  micropolygons, 5.3M samples): every sample's winner, occlZ and composited
  data, every pixel's channels and 8-bit values;
* the whole opaque 1080p frame (200,000 grids, 51.2M micropolygons, 33.2M
  samples): every pixel's channels and 8-bit values against the oracle run in
  image strips across the host cores;
* the transparent stream at a quarter of its size (480x270, 8x8 samples);
* the motion blur + depth of field stream at a tenth (192x108, 6x6 samples);
* the 640x480 sphere frame (camera-space grids, projected on the device).

Bars as in the small parity tests: winners, occlZ, fragment counts and valid
masks bit-exact; composited samples and channels within 1e-5 relative (1e-6
absolute); 8-bit values within 1 LSB.
"""
import numpy as np
import pytest

from tests.test_gpu_parity import close_or_same, compare

pytestmark = pytest.mark.gpu

QCH = (0, 1, 2, 6)
_oracle_cache = {}


def _scene(name):
    from aqsis_gb300 import scene as S
    if name == "opaque_slice":
        return S.scaled(S.opaque_stream, 0.4, seed=0xC1)
    if name == "opaque_full":
        return S.opaque_stream(seed=0xC1)
    if name == "transparent_quarter":
        return S.scaled(S.transparent_stream, 0.25, seed=0xC2)
    if name == "mbdof_tenth":
        return S.scaled(S.motion_dof_stream, 0.1, seed=0xC3)
    if name == "spheres":
        from aqsis_gb300 import spheres
        return spheres.sphere_scene(seed=0xC0)
    raise KeyError(name)


def _reference(oracle, name, strips=False):
    """The oracle's result for a named workload, computed once per session."""
    key = (name, strips)
    if key not in _oracle_cache:
        sc = _scene(name)
        ref = oracle.render_strips(sc, qchannels=QCH) if strips else oracle.render(sc, QCH)
        _oracle_cache[key] = (sc, ref)
    return _oracle_cache[key]


def _device(aqh_lib, sc, batched, samples=True):
    h = aqh_lib.Hider(0)
    try:
        h.set_mode(batched)
        h.frame_begin(sc.frame)
        h.set_samples(sc.samples)
        h.submit_grids_host(sc.grids)
        h.render(sync=True)
        res = {"channels": h.read_channels(), "quantized": h.read_quantized(QCH)}
        if samples:
            res.update(h.read_samples())
        res["stats"] = h.stats()
    finally:
        h.close()
    return res


@pytest.mark.parametrize("batched", [False, True], ids=["plain", "batched"])
def test_opaque_slice_768x432(aqh_lib, oracle, batched):
    sc, ref = _reference(oracle, "opaque_slice")
    assert sc.grids.micropolygons == 8_192_000
    res = _device(aqh_lib, sc, batched)
    compare(res, ref, exact_pixels=True)
    assert res["valid"].mean() > 0.9


def test_opaque_full_frame_1080p(aqh_lib, oracle):
    sc, ref = _reference(oracle, "opaque_full", strips=True)
    assert sc.grids.micropolygons == 51_200_000
    res = _device(aqh_lib, sc, True, samples=False)
    ca, cb = res["channels"], ref["channels"]
    assert ca.shape == (1080, 1920, 9)
    ok = close_or_same(ca, cb)
    assert ok.all(), "channels differ at %d entries" % int((~ok).sum())
    assert np.array_equal(ca.view(np.uint32), cb.view(np.uint32))
    assert np.array_equal(res["quantized"].astype(np.int64), ref["quantized"].astype(np.int64))


@pytest.mark.parametrize("batched", [False, True], ids=["plain", "batched"])
def test_transparent_quarter(aqh_lib, oracle, batched):
    sc, ref = _reference(oracle, "transparent_quarter")
    res = _device(aqh_lib, sc, batched)
    compare(res, ref)
    assert res["nfrag"].max() > 4


@pytest.mark.parametrize("batched", [False, True], ids=["plain", "batched"])
def test_motion_dof_tenth(aqh_lib, oracle, batched):
    sc, ref = _reference(oracle, "mbdof_tenth")
    res = _device(aqh_lib, sc, batched)
    compare(res, ref)


@pytest.mark.parametrize("batched", [False, True], ids=["plain", "batched"])
def test_sphere_frame_640x480(aqh_lib, oracle, batched):
    sc, ref = _reference(oracle, "spheres")
    res = _device(aqh_lib, sc, batched)
    compare(res, ref, exact_pixels=True)
