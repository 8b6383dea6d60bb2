"""CSG in the oracle (CqImagePixel::Combine's resolve, imagepixel.cpp:166-188;
csgtree.cpp:166-350): two solids made of full-screen front and back faces,
A between depths 2 and 4, B between 3 and 5, combined by union,
intersection and difference, keep the faces of the combined solid only."""
import numpy as np
import pytest

from aqsis_gb300 import scene as S
from tests import scenes_small as SS

RED, GREEN, BLUE = (1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0)


def face(z, colour, oi=None):
    n = 9 * 9
    return SS.plane(0, 0, 8, 8, z, ci=np.tile(colour, (n, 1)), oi=oi)


def solids_scene(types, parents, faces, grid_node, seed=5):
    fr = S.Frame(width=8, height=8, xsamples=2, ysamples=2, filter="box", xfilter=1.0, yfilter=1.0, q_dither=0.0)
    g = S.concat_grids([face(z, c) for z, c in faces])
    g.csg_type = np.array(types, np.int32)
    g.csg_parent = np.array(parents, np.int32)
    g.csg_node = np.array(grid_node, np.int32)
    return SS.custom(fr, g, seed=seed, explicit=True)


def inside(sc):
    x0, y0, w, h = sc.frame.sample_region
    m = np.zeros((h, w, sc.frame.spp), bool)
    m[1:-1, 1:-1] = True
    return m.reshape(-1)


A_FACES = [(2.0, RED), (4.0, RED)]
B_FACES = [(3.0, GREEN), (5.0, GREEN)]


# op node 0 over primitives 1 (A) and 2 (B); the front surviving depth and its colour
@pytest.mark.parametrize("op,first,depth,colour", [
    (S.CSG_UNION, "A", 2.0, RED),
    (S.CSG_INTERSECTION, "A", 3.0, GREEN),
    (S.CSG_DIFFERENCE, "A", 2.0, RED),       # A - B: A's front face
    (S.CSG_DIFFERENCE, "B", 4.0, RED),       # B - A: A's back face, seen inside B
])
def test_two_solids(oracle, op, first, depth, colour):
    faces = A_FACES + B_FACES
    a, b = (1, 2) if first == "A" else (2, 1)
    sc = solids_scene([op, 0, 0], [-1, 0, 0], faces, [a, a, b, b])
    res = oracle.render(sc)
    m = inside(sc)
    sd = res["sdata"].reshape(-1, 7)[m]
    assert (res["valid"][m] == 1).all()
    assert np.allclose(sd[:, 6], depth)
    assert np.allclose(sd[:, :3], colour)


def test_disjoint_intersection_leaves_samples_unwritten(oracle):
    faces = [(2.0, RED), (3.0, RED), (4.0, GREEN), (5.0, GREEN)]
    sc = solids_scene([S.CSG_INTERSECTION, 0, 0], [-1, 0, 0], faces, [1, 1, 2, 2])
    res = oracle.render(sc)
    m = inside(sc)
    assert (res["valid"][m] == 0).all()
    assert np.allclose(res["channels"].reshape(8, 8, -1)[2:-2, 2:-2, :4], 0.0)


def test_plain_grid_in_front_is_kept(oracle):
    """A grid outside any solid takes no part in the resolve."""
    faces = A_FACES + B_FACES + [(1.0, BLUE)]
    sc = solids_scene([S.CSG_INTERSECTION, 0, 0], [-1, 0, 0], faces, [1, 1, 2, 2, -1])
    res = oracle.render(sc)
    sd = res["sdata"].reshape(-1, 7)[inside(sc)]
    assert np.allclose(sd[:, 6], 1.0) and np.allclose(sd[:, :3], BLUE)


def test_nested_tree(oracle):
    """union(intersection(A, B), C) with C between 6 and 7: the
    intersection's front face (B at 3) is in front."""
    faces = A_FACES + B_FACES + [(6.0, BLUE), (7.0, BLUE)]
    types = [S.CSG_UNION, S.CSG_INTERSECTION, 0, 0, 0]
    parents = [-1, 0, 1, 1, 0]
    sc = solids_scene(types, parents, faces, [2, 2, 3, 3, 4, 4])
    res = oracle.render(sc)
    sd = res["sdata"].reshape(-1, 7)[inside(sc)]
    assert np.allclose(sd[:, 6], 3.0) and np.allclose(sd[:, :3], GREEN)
    # without the tree every face is an ordinary opaque hit: A's front wins
    sc.grids.csg_node = None
    sd = oracle.render(sc)["sdata"].reshape(-1, 7)[inside(sc)]
    assert np.allclose(sd[:, 6], 2.0) and np.allclose(sd[:, :3], RED)


def test_primitive_solid_keeps_its_faces(oracle):
    """A solid that is one primitive (a tree of one node) releases its hits
    unchanged."""
    sc = solids_scene([0], [-1], A_FACES, [0, 0])
    sd = oracle.render(sc)["sdata"].reshape(-1, 7)[inside(sc)]
    assert np.allclose(sd[:, 6], 2.0) and np.allclose(sd[:, :3], RED)


def test_two_trees(oracle):
    """Two separate solids, each resolved by its own tree: intersection(A, B)
    gives B's front at 3; difference(C, D) with C 2.5-6, D 1-7 is empty."""
    faces = A_FACES + B_FACES + [(2.5, BLUE), (6.0, BLUE), (1.0, RED), (7.0, RED)]
    types = [S.CSG_INTERSECTION, 0, 0, S.CSG_DIFFERENCE, 0, 0]
    parents = [-1, 0, 0, -1, 3, 3]
    sc = solids_scene(types, parents, faces, [1, 1, 2, 2, 4, 4, 5, 5])
    sd = oracle.render(sc)["sdata"].reshape(-1, 7)[inside(sc)]
    assert np.allclose(sd[:, 6], 3.0) and np.allclose(sd[:, :3], GREEN)


def test_random_trees_run(oracle):
    base = SS.transparent_small(seed=31, scale=0.02)
    sc = S.with_csg(base, seed=3)
    res = oracle.render(sc)
    assert np.isfinite(res["channels"][..., :4]).all()
    assert not np.array_equal(res["channels"][..., :4], oracle.render(base)["channels"][..., :4])


def test_scene_file_keeps_trees(tmp_path):
    sc = S.with_csg(SS.opaque_small(seed=32, scale=0.01), seed=4)
    p = tmp_path / "csg.npz"
    S.save_scene(str(p), sc)
    sc2, _ = S.load_scene(str(p))
    for k in ("csg_node", "csg_type", "csg_parent"):
        assert np.array_equal(getattr(sc2.grids, k), getattr(sc.grids, k))
