"""The oracle's inverse bilinear lookup against the reference's known-answer
cases (libs/core/bilinear_test.cpp:67-261): bilerp a (u,v), invert, and
expect the (u,v) back within the tolerances the reference's tests use."""
import numpy as np
import pytest

E = 1e-6
UV = [(0.5, 0.5), (0.12345, 0.67891), (0.42042, 0.42042), (0.3141592, 0.2718281),
      (0, 0), (1, 0), (0, 1), (1, 1),
      (E, E), (1 - E, E), (E, 1 - E), (1 - E, 1 - E),
      (0.5, 0), (0.5, 1), (0, 0.5), (1, 0.5),
      (0.5, E), (0.5, 1 - E), (E, 0.5), (1 - E, 0.5)]


def fixture_uv(u_ex=-1.0, v_ex=-1.0):
    """bilinear_test.cpp:104-146: optionally drop points near u = u_ex or v = v_ex."""
    out = []
    for u, v in UV:
        u32, v32 = np.float32(u), np.float32(v)
        if (u_ex == -1 or abs(np.float32(u_ex) - u32) > 1e-2) and (v_ex == -1 or abs(np.float32(v_ex) - v32) > 1e-2):
            out.append((u32, v32))
    return np.array(out, np.float32)


def close(a, b, rel, ab):
    d = np.abs(a - b)
    return (d < ab) | (d < rel * np.abs(a)) | (d < rel * np.abs(b))


OFF = (1000.0, 2000.0)
CASES = [
    # name, quad A B C D, uv fixture exclusions, rel tol, abs tol
    ("convex_irregular", [(0.1, 0.1), (1.1, 0), (-0.1, 1.5), (1, 1)], (-1, -1), 1e-3, 1e-3),
    ("convex_irregular_rot90", [(-0.1, 1.5), (0.1, 0.1), (1, 1), (1.1, 0)], (-1, -1), 1e-3, 1e-3),
    ("convex_irregular_rot180", [(1, 1), (-0.1, 1.5), (1.1, 0), (0.1, 0.1)], (-1, -1), 1e-3, 1e-3),
    ("convex_irregular_rot270", [(1.1, 0), (1, 1), (0.1, 0.1), (-0.1, 1.5)], (-1, -1), 1e-3, 1e-3),
    ("large_offset", [(0 + OFF[0], 0 + OFF[1]), (2 + OFF[0], 0 + OFF[1]), (0 + OFF[0], 1 + OFF[1]),
                      (2 + OFF[0], 1 + OFF[1])], (-1, -1), 1e-3, 1e-3),
    ("exactly_rectangular", [(0, 0), (2, 0), (0, 1), (2, 1)], (-1, -1), 1e-3, 1e-3),
    ("almost_rectangular", [(0.0001, 0.000005), (2, 0), (0, 1), (2, 1)], (-1, -1), 2e-4, 1e-4),
    ("degenerate_u_verts", [(0, 0), (0, 0), (0, 1), (1, 1.5)], (-1, 0), 1e-3, 1e-3),
    ("degenerate_u_verts2", [(0, 0), (1.1, 0), (0, 1), (0, 1)], (-1, 1), 1e-3, 1e-3),
    ("degenerate_v_verts", [(0, 0), (1, 0), (0, 0), (1, 1.5)], (0, -1), 1e-3, 1e-3),
    ("parallel_adjacent_edges_a", [(0, 0), (1, 0), (1, 1.5), (2, 0.01)], (1, 0), 0.03, 0.03),
    ("parallel_adjacent_edges_b", [(0, 0), (1, 0), (1, 1.5), (2, 0.01)], (-1, -1), 0.2, 0.2),
]


def quad_array(q):
    a = np.array(q, np.float64).reshape(8)
    return a.astype(np.float32)


@pytest.mark.parametrize("name,quad,ex,rel,ab", CASES, ids=[c[0] for c in CASES])
def test_oracle_invbilinear_known_answers(oracle, name, quad, ex, rel, ab):
    q = quad_array(quad)
    uv_in = fixture_uv(*ex)
    P = oracle.bilerp2(q, uv_in)
    uv_out = oracle.invbilinear(q, P)
    ok = close(uv_in, uv_out, np.float32(rel), np.float32(ab)).all(axis=1)
    assert ok.all(), (name, uv_in[~ok], uv_out[~ok])
    # checkLookup also bounds u to [-absTol, 1+absTol]
    assert (uv_out[:, 0] >= -np.float32(ab)).all() and (uv_out[:, 0] <= 1 + np.float32(ab)).all()
