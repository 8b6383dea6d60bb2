"""Shade / Split culling in the oracle (micropolygon.cpp:431-506, 957-1020,
1075-1080): back-facing first vertices drop their micropolygons (N flips
Ng), a static grid's trailing run of black Oi goes unless zthreshold is
black, and a moving grid needs every key facing away."""
import dataclasses

import numpy as np

from aqsis_gb300 import scene as S
from oracle import oracle as O
from tests import scenes_small as SS


def one_grid(P, nkeys=1):
    cu = cv = 2
    nv = 9
    Pk = np.zeros((nv * nkeys, 4), np.float32)
    Pk[:, :3] = P
    return S._pack(np.array([cu]), np.array([cv]), np.array([nkeys]), np.array([S.GRID_CAMERA]),
                   Pk, np.ones((nv, 4), np.float32), np.ones((nv, 4), np.float32),
                   np.linspace(0, 1, nkeys).astype(np.float32) if nkeys > 1 else None,
                   np.array([0], np.int32) if nkeys > 1 else None)


def cull(g, flags, Ng, N=None, Oi=None, zblack=0):
    L = O.lib()
    out = np.zeros(g.micropolygons, np.uint8)
    P = np.ascontiguousarray(g.P, np.float32)
    Ng = np.ascontiguousarray(Ng, np.float32)
    N = None if N is None else np.ascontiguousarray(N, np.float32)
    Oi = None if Oi is None else np.ascontiguousarray(Oi, np.float32)
    L.orc_cull_grid(int(g.cu[0]), int(g.cv[0]), int(g.nkeys[0]), flags, O._p(P, O._f32p), O._p(Ng, O._f32p),
                    O._p(N, O._f32p), O._p(Oi, O._f32p), zblack, out.ctypes.data_as(O._u8p))
    return out


def test_back_faces():
    P = np.tile([0.0, 0.0, 5.0], (9, 1))
    Ng = np.tile([0.0, 0.0, -1.0], (9, 1))      # towards the eye: kept
    Ng[0] = [0.0, 0.0, 1.0]                     # vertex 0 (micropolygon 0) faces away
    Ng[4] = [0.0, 1.0, 0.0]                     # P . Ng == 0 counts as facing away
    g = one_grid(P)
    assert list(cull(g, S.GRID_CULL_BACKFACING, Ng)) == [1, 0, 0, 1]
    N = -Ng                                     # N disagrees everywhere: Ng flips
    assert list(cull(g, S.GRID_CULL_BACKFACING, Ng, N)) == [0, 1, 1, 1]
    assert list(cull(g, 0, Ng)) == [0, 0, 0, 0]


def test_trailing_black_opacity():
    g = one_grid(np.tile([0.0, 0.0, 5.0], (9, 1)))
    Oi = np.ones((9, 4), np.float32)
    Oi[4:, :3] = 0.0                            # vertices 4..8 black: micropolygon 3 (first vertex 4)
    Oi[1, :3] = 0.0                             # not trailing: kept
    Ng = np.tile([0.0, 0.0, -1.0], (9, 1))
    assert list(cull(g, S.GRID_CULL_TRANSPARENT, Ng, Oi=Oi)) == [0, 0, 0, 1]
    assert list(cull(g, S.GRID_CULL_TRANSPARENT, Ng, Oi=Oi, zblack=1)) == [0, 0, 0, 0]


def test_motion_needs_every_key():
    P = np.tile([0.0, 0.0, 5.0], (18, 1))
    Ng = np.tile([0.0, 0.0, 1.0], (18, 1))      # both keys face away
    Ng[9 + 1] = [0.0, 0.0, -1.0]                # vertex 1 faces the eye at key 1
    g = one_grid(P, nkeys=2)
    assert list(cull(g, S.GRID_CULL_BACKFACING, Ng)) == [1, 0, 1, 1]
    Oi = np.zeros((9, 4), np.float32)           # no opacity culling on moving grids
    assert list(cull(g, S.GRID_CULL_TRANSPARENT, Ng, Oi=Oi)) == [0, 0, 0, 0]


def test_random_culling_culls():
    base = SS.camera_small(seed=61, every=1)
    sc = S.with_culling(base, seed=1)
    a = O.render(base)["winner"] >= 0
    b = O.render(sc)["winner"] >= 0
    assert b.sum() < a.sum()


def test_scene_file_keeps_normals(tmp_path):
    sc = S.with_culling(SS.camera_small(seed=62, every=1), seed=2)
    p = tmp_path / "cull.npz"
    S.save_scene(str(p), sc)
    sc2, _ = S.load_scene(str(p))
    assert np.array_equal(sc2.grids.cull_Ng, sc.grids.cull_Ng)
