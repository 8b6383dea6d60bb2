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


def fuzz(seed):
    """A small random frame for differential tests: random pixel samples,
    filter, crop window, depth filter, zthreshold and dither; grids of random
    size and placement with jitter, exact depth ties, collapsed vertices,
    mirrored (clockwise) grids, z at and below zero, huge quads, constant and
    smooth shading, matte flags, transparency (including Oi of 0 and above
    1), triangular grids, culled micropolygons and, for some seeds, motion
    and depth of field."""
    rng = np.random.default_rng(1000 + seed)
    filters = [("box", 1.0, 1.0), ("gaussian", 2.0, 2.0), ("catmull-rom", 3.0, 3.0), ("triangle", 2.0, 2.0),
               ("sinc", 4.0, 4.0), ("gaussian", 3.0, 1.0)]
    filt = filters[int(rng.integers(0, len(filters)))]
    w, h = int(rng.integers(12, 48)), int(rng.integers(10, 40))
    crop = None
    if rng.random() < 0.3:
        x0, y0 = int(rng.integers(0, w // 2)), int(rng.integers(0, h // 2))
        crop = (x0, int(rng.integers(x0 + 1, w + 1)), y0, int(rng.integers(y0 + 1, h + 1)))
    motion = rng.random() < 0.25
    dof = rng.random() < 0.2
    fr = S.Frame(width=w, height=h, crop=crop, xsamples=int(rng.integers(1, 7)), ysamples=int(rng.integers(1, 7)),
                 filter=filt[0], xfilter=filt[1], yfilter=filt[2], q_dither=float(rng.choice([0.0, 0.5])),
                 depth_filter=int(rng.choice([0, 0, 0, 1, 2, 3])),
                 zthreshold=tuple(float(v) for v in rng.choice([1.0, 0.5], 3)),
                 display_z=int(rng.random() < 0.2))
    if motion:
        fr.shutter = (0.0, 1.0)
    if dof:
        fr.fstop, fr.focal_length, fr.focal_distance = 2.8, 0.5, 20.0
    parts = []
    for k in range(int(rng.integers(3, 14))):
        nx, ny = int(rng.integers(1, 9)), int(rng.integers(1, 9))
        step = float(rng.choice([0.4, 1.0, 1.7, 6.0]))
        z = float(rng.choice([rng.uniform(0.5, 60), 20.0, 0.0, -3.0], p=[0.7, 0.2, 0.05, 0.05]))

        oi = None
        r = rng.random()
        if r < 0.3:
            oi = rng.uniform(0.0, 1.2, ((nx + 1) * (ny + 1), 3))
        elif r < 0.35:
            oi = np.zeros(((nx + 1) * (ny + 1), 3))
        flags = int(rng.choice([S.GRID_SMOOTH, 0, S.GRID_SMOOTH | S.GRID_MATTE, S.GRID_MATTEALPHA | S.GRID_SMOOTH],
                               p=[0.6, 0.25, 0.1, 0.05]))
        g = plane(float(rng.uniform(-4, w)), float(rng.uniform(-4, h)), nx, ny, z, step=step, rng=rng,
                  jitter=float(rng.choice([0.0, 0.3])), oi=oi, flags=flags,
                  zslope=float(rng.choice([0.0, 0.02, -0.05])))
        P = g.P.reshape(ny + 1, nx + 1, 4).copy()
        if rng.random() < 0.2:
            P = P[:, ::-1, :].copy()                       # clockwise
        if rng.random() < 0.2 and nx > 1:
            i, j = int(rng.integers(0, ny + 1)), int(rng.integers(0, nx))
            P[i, j + 1, :3] = P[i, j, :3]                  # collapsed edge
        g = grid_from_points(P[..., :3], g.Ci[:, :3], None if oi is None else np.asarray(oi), flags)
        if rng.random() < 0.15:
            g.flags = (g.flags | S.GRID_TRIANGULAR).astype(np.int32)
        if motion and rng.random() < 0.6:
            d = rng.uniform(-4, 4, 2).astype(np.float32)
            P1 = g.P.copy()
            P1[:, 0] += d[0]
            P1[:, 1] += d[1]
            g = S._pack(g.cu, g.cv, np.array([2]), g.flags, np.concatenate([g.P, P1]), g.Ci, g.Oi,
                        np.array([0.0, 1.0], np.float32), np.array([0]))
        parts.append(g)
    grids = S.concat_grids(parts)
    if dof:
        # a vertex at camera depth 0 has an infinite circle of confusion; the
        # reference's integer conversions of the infinite bounds are undefined
        # (and differ between hosts), so no parity is defined for it
        z = grids.P[:, 2]
        z[z == 0.0] = 1e-3
    if rng.random() < 0.3:
        culled = np.zeros(grids.micropolygons, np.uint8)
        culled[rng.integers(0, grids.micropolygons, max(1, grids.micropolygons // 10))] = 1
        grids.culled = culled
    sc = custom(fr, grids, seed=seed, dither=fr.q_dither > 0)
    if rng.random() < 0.25:
        sc = S.with_lod(sc, seed=seed)
    return sc


def motion_static_behind_eye(seed=16, transparent=False):
    """A motion-blurred frame with a static grid at negative camera depth
    beside a moving one.  Only micropolygons that move (or see depth of
    field) go through RenderMPG_MBOrDof and its clipping-range cull; the
    static grid is sampled like any static one."""
    rng = np.random.default_rng(seed)
    fr = S.Frame(width=28, height=24, xsamples=3, ysamples=3, filter="gaussian", xfilter=2.0, yfilter=2.0,
                 q_dither=0.0, shutter=(0.0, 1.0))
    oi = rng.uniform(0.2, 0.8, (49, 3)) if transparent else None
    still = plane(2, 3, 6, 6, -4.0, step=2.0, rng=rng, jitter=0.3, zslope=0.01, oi=oi)
    mov = plane(10, 6, 6, 6, 20.0, step=1.5, rng=rng, jitter=0.2)
    P1 = mov.P.copy()
    P1[:, 0] += 3.0
    P1[:, 1] -= 1.5
    mov = S._pack(mov.cu, mov.cv, np.array([2]), mov.flags, np.concatenate([mov.P, P1]), mov.Ci, mov.Oi,
                  np.array([0.0, 1.0], np.float32), np.array([0]))
    return custom(fr, S.concat_grids([still, mov]), seed=seed)
