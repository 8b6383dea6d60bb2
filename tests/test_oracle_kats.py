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
