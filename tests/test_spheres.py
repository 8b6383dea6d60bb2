"""The sphere scene generator (dicing and shading restated from the
reference's quadric and plastic code): grid sizes, micropolygon sizes after
Split's projection, and an oracle frame of it."""
import numpy as np
import pytest

from aqsis_gb300 import scene as S
from aqsis_gb300 import spheres


@pytest.fixture(scope="module")
def small():
    return spheres.sphere_scene(seed=3, nspheres=6, width=160, height=120)


def test_grids_are_diced_to_the_grid_size(small):
    g = small.grids
    assert g.ngrids > 0
    assert (g.cu >= 1).all() and (g.cu <= spheres.GRID_SIDE).all()
    assert (g.cv >= 1).all() and (g.cv <= spheres.GRID_SIDE).all()
    assert (g.flags & S.GRID_CAMERA).all() and (g.flags & S.GRID_OPAQUE).all()
    assert small.frame.camera_to_raster is not None


def test_micropolygons_are_about_a_pixel(oracle, small):
    g = oracle.projected_grids(small)
    edges = []
    for i in range(g.ngrids):
        cu, cv = int(g.cu[i]), int(g.cv[i])
        P = g.P[int(g.pbase[i]):int(g.pbase[i]) + (cu + 1) * (cv + 1), :2].reshape(cv + 1, cu + 1, 2)
        edges.append(np.linalg.norm(P[:, 1:] - P[:, :-1], axis=-1).ravel())
        edges.append(np.linalg.norm(P[1:] - P[:-1], axis=-1).ravel())
    e = np.concatenate(edges)
    # EstimateGridSize aims at the shading rate (1 pixel) for the longest edge of the estimate grid
    assert np.median(e) < 1.0
    assert e.max() < 2.5


def test_oracle_frame_of_spheres(oracle, small):
    res = oracle.render(small)
    assert res["valid"].mean() > 0.02
    q = res["quantized"]
    assert q.max() > 0
