"""Small seeded scenes for parity tests: the benchmark generators at reduced
size plus hand-built edge cases (degenerate and clockwise micropolygons,
coplanar ties, culled micropolygons, large quads spanning tiles, crop windows,
constant shading, matte objects, odd pixel-sample counts)."""
import numpy as np

from aqsis_gb300 import scene as S


def custom(frame, grids, seed=7, explicit=False, npatterns=64, dither=False):
    rng = np.random.default_rng(seed)
    return S.Scene(frame, grids, S.make_samples(frame, rng, npatterns, explicit, dither))


def grid_from_points(P, Ci=None, Oi=None, flags=S.GRID_SMOOTH, cu=None, cv=None):
    """One grid from a (cv+1, cu+1, 3) point array."""
    P = np.asarray(P, np.float32)
    cv1, cu1 = P.shape[:2]
    n = cv1 * cu1
    P4 = np.zeros((n, 4), np.float32)
    P4[:, :3] = P.reshape(n, 3)
    C4 = np.zeros((n, 4), np.float32)
    O4 = np.ones((n, 4), np.float32)
    O4[:, 3] = 0
    if Ci is not None:
        C4[:, :3] = np.asarray(Ci, np.float32).reshape(n, 3)
    else:
        C4[:, :3] = 1.0
    opaque = True
    if Oi is not None:
        O4[:, :3] = np.asarray(Oi, np.float32).reshape(n, 3)
        opaque = bool((O4[:, :3] >= 1).all())
    if opaque:
        flags |= S.GRID_OPAQUE
    return S._pack(np.array([cu1 - 1]), np.array([cv1 - 1]), np.array([1]), np.array([flags]), P4, C4, O4)


def plane(x0, y0, nx, ny, z, step=1.0, rng=None, jitter=0.0, ci=None, oi=None, flags=S.GRID_SMOOTH, zslope=0.0):
    xs = x0 + np.arange(nx + 1) * step
    ys = y0 + np.arange(ny + 1) * step
    X, Y = np.meshgrid(xs, ys)
    if jitter and rng is not None:
        X = X + rng.uniform(-jitter, jitter, X.shape)
        Y = Y + rng.uniform(-jitter, jitter, Y.shape)
    Z = np.full_like(X, z) + zslope * (X - x0)
    P = np.stack([X, Y, Z], -1)
    n = (nx + 1) * (ny + 1)
    if ci is None:
        rng2 = rng if rng is not None else np.random.default_rng(1)
        ci = rng2.random((n, 3))
    return grid_from_points(P, ci, oi, flags)


def opaque_small(seed=1, explicit=False, scale=0.05):
    return S.scaled(S.opaque_stream, scale, seed=seed, explicit_samples=explicit)


def transparent_small(seed=2, scale=0.05):
    return S.scaled(S.transparent_stream, scale, seed=seed)


def edge_cases(seed=3, xs=4, ys=4, filt=("gaussian", 2.0, 2.0)):
    rng = np.random.default_rng(seed)
    fr = S.Frame(width=64, height=48, xsamples=xs, ysamples=ys, filter=filt[0], xfilter=filt[1], yfilter=filt[2],
                 q_dither=0.0)
    parts = []
    # a big jittered plane covering most of the image
    parts.append(plane(-3, -3, 35, 27, 50.0, step=2.0, rng=rng, jitter=0.4, zslope=0.01))
    # coplanar duplicate of a patch: exact depth ties, first inserted must win
    parts.append(plane(10, 10, 8, 8, 20.0, rng=np.random.default_rng(5)))
    parts.append(plane(10, 10, 8, 8, 20.0, rng=np.random.default_rng(6)))
    # clockwise grid (mirrored in x)
    g = plane(30, 5, 6, 6, 30.0, rng=rng, jitter=0.2)
    P = g.P.reshape(7, 7, 4)[:, ::-1, :].copy()
    parts.append(grid_from_points(P[..., :3], rng.random((49, 3))))
    # degenerate micropolygons: collapse some vertex pairs
    g = plane(40, 20, 5, 5, 15.0, rng=rng)
    P = g.P.reshape(6, 6, 4).copy()
    P[2, 3, :3] = P[2, 2, :3]          # A--B coincide
    P[4, 1, :3] = P[3, 1, :3]          # vertical collapse
    P[1, 4, :3] = P[1, 5, :3]
    parts.append(grid_from_points(P[..., :3], rng.random((36, 3))))
    # large micropolygons spanning several tiles
    parts.append(plane(-5, 20, 3, 2, 10.0, step=9.0, rng=rng, jitter=1.0))
    # constant shading and a matte patch
    parts.append(plane(20, 30, 6, 4, 12.0, rng=rng, flags=0))
    parts.append(plane(5, 35, 6, 4, 11.0, rng=rng, flags=S.GRID_SMOOTH | S.GRID_MATTE))
    # a non-square grid bigger than one round of micropolygons (40 x 9 = 360)
    parts.append(plane(1, 2, 40, 9, 25.0, step=1.3, rng=rng, jitter=0.3))
    # micropolygons partly outside the image and beyond the crop cull
    parts.append(plane(-10, -10, 4, 4, 5.0, step=2.5, rng=rng))
    parts.append(plane(70, 50, 3, 3, 5.0, rng=rng))
    grids = S.concat_grids(parts)
    # cull a few micropolygons
    culled = np.zeros(grids.micropolygons, np.uint8)
    culled[rng.integers(0, grids.micropolygons, 40)] = 1
    grids.culled = culled
    return custom(fr, grids, seed=seed)


def transparent_edge(seed=4, xs=3, ys=3):
    rng = np.random.default_rng(seed)
    fr = S.Frame(width=40, height=32, xsamples=xs, ysamples=ys, filter="catmull-rom", xfilter=3.0, yfilter=3.0,
                 q_dither=0.0)
    parts = [plane(-2, -2, 22, 18, 40.0, step=2.0, rng=rng, jitter=0.3)]
    for k in range(6):
        op = rng.uniform(0.1, 0.9, ((7 * 7), 3))
        parts.append(plane(rng.uniform(0, 30), rng.uniform(0, 22), 6, 6, float(rng.uniform(5, 60)), rng=rng,
                           jitter=0.3, oi=op))
    # a transparent layer exactly coplanar with an opaque one (ties with the occluding hit)
    parts.append(plane(8, 8, 5, 5, 40.0, step=2.0, rng=rng, oi=np.full((36, 3), 0.5)))
    # fully transparent-black opacity and over-unity opacity
    parts.append(plane(25, 3, 4, 4, 7.0, rng=rng, oi=np.zeros((25, 3))))
    parts.append(plane(3, 20, 4, 4, 8.0, rng=rng, oi=np.full((25, 3), 1.5)))
    return custom(fr, S.concat_grids(parts), seed=seed)


def motion_dof_small(seed=5, motion=20.0, dof=True, xs=6, ys=6, scale=0.04, transparent=False):
    """The motion blur + depth of field stream at reduced size (box 1x1)."""
    sc = S.scaled(S.motion_dof_stream, scale, seed=seed, motion=motion, dof=dof, xs=xs, ys=ys)
    if transparent:
        rng = np.random.default_rng(seed + 100)
        g = sc.grids
        g.Oi[:, :3] = rng.uniform(0.2, 0.9, (g.Oi.shape[0], 3)).astype(np.float32)
        g.flags = (g.flags & ~S.GRID_OPAQUE).astype(np.int32)
    return sc


def dof_only_small(seed=6, xs=4, ys=4, scale=0.04):
    sc = S.scaled(S.motion_dof_stream, scale, seed=seed, motion=None, dof=True, xs=xs, ys=ys)
    return sc


def motion_mixed_small(seed=7, dof=False, xs=4, ys=4, scale=0.04):
    """A motion-blurred frame whose grids alternate between moving and
    static (one key), as a scene with a camera-fixed prop would give."""
    sc = S.scaled(S.motion_dof_stream, scale, seed=seed, motion=20.0, dof=dof, xs=xs, ys=ys)
    rng = np.random.default_rng(seed + 200)
    fr = sc.frame
    n = max(4, sc.grids.ngrids // 2)
    moving = S.regular_grids(n, fr.width, fr.height, rng, motion=20.0)
    still = S.regular_grids(n, fr.width, fr.height, rng)
    parts = []
    for k in range(0, n, 8):
        parts.append(_take(moving, k, min(n, k + 8)))
        parts.append(_take(still, k, min(n, k + 8)))
    sc.grids = S.concat_grids(parts)
    return sc


def _take(g, a, b):
    """Grids [a, b) of a packed stream as their own stream."""
    nv = (g.cu.astype(np.int64) + 1) * (g.cv.astype(np.int64) + 1)
    p0, p1 = int(g.pbase[a]), int(g.pbase[b - 1] + nv[b - 1] * g.nkeys[b - 1])
    c0, c1 = int(g.cbase[a]), int(g.cbase[b - 1] + nv[b - 1])
    t0 = int(g.tbase[a])
    t1 = int(g.tbase[b - 1] + g.nkeys[b - 1]) if len(g.times) > 1 else 1
    sub = S._pack(g.cu[a:b], g.cv[a:b], g.nkeys[a:b], g.flags[a:b], g.P[p0:p1], g.Ci[c0:c1], g.Oi[c0:c1],
                  g.times[t0:t1], (g.tbase[a:b] - t0))
    return sub


def transparent_hidden_occluder(seed=8, xs=4, ys=4):
    """Transparent grids plus a grid not flagged opaque whose opacity is 1 on
    every vertex: its micropolygons occlude (SqMpgSampleInfo::isOpaque), so
    the frame must take the ordered path although no grid says so."""
    rng = np.random.default_rng(seed)
    fr = S.Frame(width=40, height=32, xsamples=xs, ysamples=ys, filter="gaussian", xfilter=2.0, yfilter=2.0,
                 q_dither=0.0)
    parts = []
    for k in range(5):
        op = rng.uniform(0.2, 0.8, (49, 3))
        parts.append(plane(rng.uniform(0, 30), rng.uniform(0, 22), 6, 6, float(rng.uniform(5, 60)), rng=rng,
                           jitter=0.3, oi=op))
    occ = plane(6, 6, 20, 14, 30.0, step=1.3, rng=rng, jitter=0.2)
    occ.flags = (occ.flags & ~S.GRID_OPAQUE).astype(np.int32)   # opaque by value, not by flag
    parts.insert(2, occ)
    return custom(fr, S.concat_grids(parts), seed=seed)


def triangular(sc, every=3):
    """Mark every `every`-th grid of a scene triangular (fTriangular: the far
    half of each grid, behind the line through corners cu and cv*(cu+1), is
    not drawn)."""
    g = sc.grids
    f = g.flags.copy()
    f[::every] |= S.GRID_TRIANGULAR
    g.flags = f.astype(np.int32)
    return sc


def triangular_small(seed=9):
    return triangular(edge_cases(seed=seed))


def triangular_motion_small(seed=10, dof=True):
    return triangular(motion_dof_small(seed=seed, dof=dof, xs=4, ys=4, scale=0.03), every=2)


def triangular_transparent_small(seed=11):
    return triangular(transparent_small(seed=seed, scale=0.03), every=2)


def camera_small(seed=14, every=2, **kw):
    """Opaque stream with every `every`-th grid given in camera space
    (GRID_CAMERA) under a perspective camera-to-raster matrix."""
    return S.to_camera_space(opaque_small(seed=seed), every=every, **kw)
