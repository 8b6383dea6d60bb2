"""Known-answer tests that pin the oracle's building blocks to values fixed
outside this repository.

* Rounding helpers: the reference's own cases for lfloor / lceil / lround
  (libs/math/math_test.cpp:36-62).  The hider uses them for sample ranges,
  filter widths and the quantize step (ddmanager.cpp:1068).
* MT19937 (libs/math/random.cpp, the global generator behind the sample
  patterns and the quantize dither): the 10000th output after seeding with
  5489 is 4123659995 (the value ISO C++ requires of std::mt19937), and the
  first outputs for the reference's seeds 545 and 19 equal numpy's legacy
  MT19937 (an independent implementation seeded by the same init_genrand).
* Filter functions (filters.cpp): values worked out by hand from the RI
  formulas at points where they are exact or have a closed form.
"""
import math

import numpy as np
import pytest


@pytest.mark.parametrize("x,want", [(1.0, 1), (-1.0, -1), (1.1, 1), (-1.1, -2)])
def test_lfloor_reference_cases(oracle, x, want):
    assert oracle.lib().orc_lfloor(x) == want


@pytest.mark.parametrize("x,want", [(1.0, 1), (-1.0, -1), (1.1, 2), (-1.1, -1)])
def test_lceil_reference_cases(oracle, x, want):
    assert oracle.lib().orc_lceil(x) == want


@pytest.mark.parametrize("x,want", [(1.0, 1), (1.2, 1), (1.5, 2), (1.7, 2),
                                    (-1.0, -1), (-1.2, -1), (-1.5, -1), (-1.7, -2)])
def test_lround_reference_cases(oracle, x, want):
    # lround<float>: x - 0.5 is evaluated in double (math.h:67-70)
    assert oracle.lib().orc_lround(float(np.float32(x))) == want


def test_vector2d_magnitudes(oracle):
    """CqVector2D::Magnitude and Magnitude2 of (0.3, 0.4): the reference's own
    known answers, checked for exact float equality
    (libs/math/vector2d_test.cpp:48-60).  0.3f^2 + 0.4f^2 lies exactly halfway
    between two floats and rounds to the even one, 0.25."""
    L = oracle.lib()
    assert L.orc_mag2(0.3, 0.4) == np.float32(0.25)
    assert L.orc_mag(0.3, 0.4) == np.float32(0.5)
    # the zero-component branches (vector2d.h:134-137, 143-146)
    assert L.orc_mag2(0.0, 0.4) == np.float32(0.4) * np.float32(0.4)
    assert L.orc_mag(-0.3, 0.0) == np.float32(0.3)


def test_mt19937_iso_value(oracle):
    L = oracle.lib()
    L.orc_mt_seed(5489)
    v = 0
    for _ in range(10000):
        v = L.orc_mt_int32()
    assert v == 4123659995


@pytest.mark.parametrize("seed", [545, 19, 5489])
def test_mt19937_matches_independent_generator(oracle, seed):
    L = oracle.lib()
    L.orc_mt_seed(seed)
    ours = np.array([L.orc_mt_int32() for _ in range(1500)], np.uint64)
    theirs = np.random.RandomState(seed)._bit_generator.random_raw(1500)
    assert np.array_equal(ours, theirs)


def test_mt_float_scale(oracle):
    # random.cpp: RandomFloat = genrand_int32 * (1 / 4294967424.0), always < 1
    L = oracle.lib()
    L.orc_mt_seed(545)
    ints = np.random.RandomState(545)._bit_generator.random_raw(200)
    got = np.array([L.orc_mt_float() for _ in range(200)], np.float32)
    want = (ints.astype(np.float64) * (1.0 / 4294967424.0)).astype(np.float32)
    assert np.array_equal(got, want)
    assert got.max() < 1.0


FILTER_CASES = [
    # (filter, x, y, xw, yw, value)
    ("gaussian", 0.0, 0.0, 2.0, 2.0, 1.0),
    ("gaussian", 0.5, 0.0, 2.0, 2.0, math.exp(-0.5)),
    ("gaussian", 0.5, 0.5, 2.0, 2.0, math.exp(-1.0)),
    ("box", 0.5, 0.5, 1.0, 1.0, 1.0),
    ("box", 0.6, 0.0, 1.0, 1.0, 0.0),
    ("triangle", 0.5, 0.0, 2.0, 2.0, 0.5),
    ("triangle", 0.0, 1.5, 2.0, 2.0, 0.0),
    ("catmull-rom", 0.0, 0.0, 3.0, 3.0, 2.0),
    ("catmull-rom", 0.5, 0.0, 3.0, 3.0, 1.125),
    ("catmull-rom", 1.0, 0.0, 3.0, 3.0, 0.0),
    ("catmull-rom", 1.5, 0.0, 3.0, 3.0, -0.125),
    ("catmull-rom", 2.0, 0.0, 3.0, 3.0, 0.0),
    ("sinc", 0.0, 0.0, 4.0, 4.0, 1.0),
    ("sinc", 1.0, 0.0, 4.0, 4.0, 0.0),
    ("disk", 0.4, 0.0, 1.0, 1.0, 1.0),
    ("disk", 0.5, 0.0, 1.0, 1.0, 0.0),
]


@pytest.mark.parametrize("name,x,y,xw,yw,want", FILTER_CASES)
def test_filter_functions(oracle, name, x, y, xw, yw, want):
    from aqsis_gb300.scene import FILTERS
    got = oracle.lib().orc_filter_eval(FILTERS[name], x, y, xw, yw)
    assert abs(got - want) <= 1e-6 * max(1.0, abs(want)), (name, got, want)


def test_filter_table_zero_outside_window(oracle):
    # InitialiseFilterValues: weights are 0 outside +-ceil(w)/2 (bucketprocessor.cpp:846-851)
    from aqsis_gb300.scene import FILTERS
    t = oracle.filter_table(FILTERS["gaussian"], 2.0, 2.0, 4, 4).reshape(3, 3, 4, 4)
    # pixel offset (-1,-1), sub-pixel (0,0): centre at (-1.375, -1.375) -> outside +-1
    assert t[0, 0, 0, 0] == 0.0
    assert t[1, 1].min() > 0.0


def test_projection_follows_matrix_vector_product(oracle):
    """orc_project_points against CqMatrix::operator*(CqVector3D)
    (matrix.h:717-750) written out in float32 steps: row-vector products,
    x and y times 1/h only when h != 1, the camera z kept."""
    from aqsis_gb300 import scene as S
    f32 = np.float32
    rng = np.random.default_rng(3)
    pts = np.zeros((400, 4), np.float32)
    pts[:, 0] = rng.uniform(-50, 50, 400)
    pts[:, 1] = rng.uniform(-50, 50, 400)
    pts[:, 2] = rng.uniform(0.5, 900, 400)
    pts[:5, 2] = 1.0                      # h == 1 under the perspective matrix: no divide
    pts[5, 2] = -3.0                      # behind the eye: negative h
    pts[:, 3] = rng.uniform(0, 1, 400)    # carried through
    for m in (S.camera_to_raster(64, 48), S.camera_to_raster(64, 48, orthographic=True),
              tuple(rng.uniform(-2, 2, 16).astype(np.float32))):
        mm = np.asarray(m, np.float32)
        got = oracle.project_points(mm, pts)
        for i in range(pts.shape[0]):
            x, y, z, w = (f32(v) for v in pts[i])
            h = f32(f32(f32(mm[3] * x) + f32(mm[7] * y)) + f32(mm[11] * z)) + mm[15]
            rx = f32(f32(f32(mm[0] * x) + f32(mm[4] * y)) + f32(mm[8] * z)) + mm[12]
            ry = f32(f32(f32(mm[1] * x) + f32(mm[5] * y)) + f32(mm[9] * z)) + mm[13]
            if h != f32(1):
                inv = f32(1) / f32(h)
                rx, ry = f32(rx * inv), f32(ry * inv)
            want = np.array([rx, ry, z, w], np.float32)
            assert np.array_equal(got[i].view(np.uint32), want.view(np.uint32)), (i, got[i], want)


def test_camera_space_scene_projects_back(oracle):
    """Split's projection of a scene unprojected by to_camera_space lands on
    the raster points within float rounding and keeps z bit for bit."""
    from aqsis_gb300 import scene as S
    from tests import scenes_small as SS
    sc = SS.opaque_small(seed=5)
    cs = S.to_camera_space(sc, every=3)
    g = oracle.projected_grids(cs)
    assert not (g.flags & S.GRID_CAMERA).any()
    assert np.array_equal(g.P[:, 2], sc.grids.P[:, 2])
    assert np.abs(g.P[:, :2] - sc.grids.P[:, :2]).max() < 1e-3
