"""The float path's rounding error against the oracle's float64 twin of
Combine and the filter (composite, filter sums, normalisation and exposure
re-evaluated in double from the same per-sample entries), per fixture scene.

The device matches the oracle bit for bit on these scenes (tests/
test_golden.py on the GPU), so the figures are the device's too.  Bars: the
colour, opacity, alpha and coverage channels within 1e-4 relative and 1e-5
absolute of double precision, depths within 1e-5 relative; a float depth
sum that overflows where the double one does not (FLT_MAX depths under
negative filter lobes, as in the reference's float path) is counted, not
compared."""
import glob
import os

import pytest

from aqsis_gb300 import scene as S

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = [p for p in sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
            if "reference_patterns" not in p]


def fp64_errors(oracle, scene):
    r = oracle.render(scene, want_fp64=True, want_samples=False)
    col = [0, 1, 2, 3, 4, 5, 6, 8]
    return (oracle.fp64_error(r["channels"][..., col], r["channels64"][..., col]),
            oracle.fp64_error(r["channels"][..., 7], r["channels64"][..., 7]))


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_float_path_against_float64(oracle, path):
    sc, _ = S.load_scene(path)
    ch, z = fp64_errors(oracle, sc)
    assert ch["max_rel"] <= 1e-4 and ch["max_abs"] <= 1e-5, ch
    assert z["max_rel"] <= 1e-5, z
