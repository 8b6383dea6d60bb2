"""Seeded micropolygon streams, frame options and sample patterns.

A ``Scene`` holds exactly what the hider consumes, in the layouts of
``include/aqh.h``: shaded grids (raster-space P plus Ci/Oi, float4 SoA), the
frame options that SqOptionCache / CqRenderer supply (libs/core/optioncache.cpp,
renderer.h), and the sample pattern caches an IqSampler hands to
CqImagePixel::setSamples (libs/core/isampler.h, imagepixel.cpp:334-359).

The generators make the workloads the benchmark configurations name:

* ``opaque_stream`` -- 16x16-quad grids in raster space, origins uniform over
  the image, vertex spacing 1 px with +-0.3 px jitter, z = z0 + s*(x - x0),
  Ci ~ U[0,1]^3, Oi = 1 (gaussian 2x2, PixelSamples 4 4 at full size).
* ``transparent_stream`` -- the same generator with Oi ~ U[0.1,0.9]^3 and grid
  origins concentrated in a centre window.
* ``motion_dof_stream`` -- two motion keys per vertex with a per-grid
  displacement, plus depth-of-field lens samples.

Inputs are synthetic stand-ins with the configured shapes, sizes and value
distributions; nothing here reads a dataset.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np

FILTERS = {"box": 0, "triangle": 1, "gaussian": 2, "catmull-rom": 3, "sinc": 4,
           "disk": 5, "bessel": 6, "mitchell": 7}
GRID_SMOOTH, GRID_MATTE, GRID_MATTEALPHA, GRID_OPAQUE, GRID_TRIANGULAR, GRID_CAMERA = 1, 2, 4, 8, 16, 32
GRID_TRIM_OUTSIDE = 64
GRID_CULL_BACKFACING, GRID_CULL_TRANSPARENT = 128, 256
FLT_MAX = float(np.finfo(np.float32).max)


@dataclasses.dataclass
class Frame:
    """Frame options (aqh_frame_desc).  Defaults are the reference's
    (libs/core/options.cpp:273-310)."""
    width: int = 640
    height: int = 480
    crop: Optional[tuple] = None          # (xmin, xmax, ymin, ymax) in pixels
    bucket: tuple = (16, 16)
    xsamples: int = 2
    ysamples: int = 2
    xfilter: float = 2.0
    yfilter: float = 2.0
    filter: str = "gaussian"
    gain: float = 1.0
    gamma: float = 1.0
    q_one: float = 255.0
    q_min: float = 0.0
    q_max: float = 255.0
    q_dither: float = 0.5
    shutter: tuple = (0.0, 0.0)
    fstop: float = FLT_MAX
    focal_length: float = 0.0
    focal_distance: float = 0.0
    dof_scale: tuple = (1.0, 1.0)
    depth_filter: int = 0
    zthreshold: tuple = (1.0, 1.0, 1.0)
    display_z: int = 0
    # camera-to-raster matrix (16 floats, CqMatrix order m[row*4 + col]) for
    # GRID_CAMERA grids, whose P is in camera space; None = no projection
    camera_to_raster: Optional[tuple] = None

    @property
    def spp(self) -> int:
        return self.xsamples * self.ysamples

    @property
    def crop_window(self) -> tuple:
        return self.crop if self.crop is not None else (0, self.width, 0, self.height)

    @property
    def shift(self) -> tuple:
        # CqBucketProcessor::m_DiscreteShiftX/Y = lfloor(filterwidth/2)
        return (int(math.floor(np.float32(self.xfilter) / np.float32(2.0))),
                int(math.floor(np.float32(self.yfilter) / np.float32(2.0))))

    @property
    def sample_region(self) -> tuple:
        """(x0, y0, w, h) of the sample region: crop window grown by the shift."""
        cx0, cx1, cy0, cy1 = self.crop_window
        sx, sy = self.shift
        return (cx0 - sx, cy0 - sy, (cx1 - cx0) + 2 * sx, (cy1 - cy0) + 2 * sy)

    @property
    def use_dof(self) -> bool:
        return 0.0 < self.fstop < FLT_MAX

    def dof_terms(self) -> tuple:
        """(m_DofMultiplier, m_OneOverFocalDistance) as CqRenderer::SetDepthOfFieldData
        computes them (renderer.h:368-377): double arithmetic stored to float."""
        if not self.use_dof:
            return (0.0, 0.0)
        lens = np.float32(np.float32(self.focal_length) / np.float32(self.fstop))
        fd = np.float32(self.focal_distance)
        mult = np.float32(0.5 * float(lens) * float(fd) / float(np.float32(fd + lens)))
        inv = np.float32(1.0 / float(fd))
        return (float(mult), float(inv))


@dataclasses.dataclass
class Grids:
    """Packed shaded grids (aqh_submit_grids_device layout)."""
    cu: np.ndarray        # int32[G]
    cv: np.ndarray        # int32[G]
    nkeys: np.ndarray     # int32[G]
    flags: np.ndarray     # int32[G]
    pbase: np.ndarray     # int64[G] first vertex of key 0 in P
    cbase: np.ndarray     # int64[G] first vertex in Ci/Oi
    tbase: np.ndarray     # int32[G] first key time
    times: np.ndarray     # float32[T]
    P: np.ndarray         # float32[NP, 4]
    Ci: np.ndarray        # float32[NC, 4]
    Oi: np.ndarray        # float32[NC, 4]
    culled: Optional[np.ndarray] = None  # uint8[total micropolygons]
    aov: Optional[np.ndarray] = None     # float32[NC, naov] output variables per vertex, indexed like Ci
    lod: Optional[np.ndarray] = None     # float32[G, 2] LevelOfDetailBounds (min, max) per grid
    csg_node: Optional[np.ndarray] = None    # int32[G] primitive CSG node of each grid, -1 = none
    csg_type: Optional[np.ndarray] = None    # int32[N] CSG node types (GRID_CSG_*)
    csg_parent: Optional[np.ndarray] = None  # int32[N] parent node, -1 = a root
    trim_set: Optional[np.ndarray] = None    # int32[G] trim set of each grid, -1 = not trimmable
    trim_uv: Optional[np.ndarray] = None     # float32[NC, 2] surface (u, v) per vertex, indexed like Ci
    trim_points: Optional[np.ndarray] = None      # float32[NPTS, 2] prepared trim-curve points
    trim_loop_first: Optional[np.ndarray] = None  # int32[NLOOPS + 1] first point of each loop
    trim_set_first: Optional[np.ndarray] = None   # int32[NSETS + 1] first loop of each set
    cull_Ng: Optional[np.ndarray] = None  # float32[NP, 3] camera-space geometric normal per P entry (every key)
    cull_N: Optional[np.ndarray] = None   # float32[NP, 3] shading normal per P entry, or None

    @property
    def ngrids(self) -> int:
        return int(self.cu.shape[0])

    @property
    def micropolygons(self) -> int:
        return int(np.sum(self.cu.astype(np.int64) * self.cv.astype(np.int64)))

    def nbytes_algorithmic(self) -> int:
        """P per key plus Ci and Oi per vertex, float4 each, read once."""
        nv = (self.cu.astype(np.int64) + 1) * (self.cv.astype(np.int64) + 1)
        return int(np.sum(nv * (16 * self.nkeys.astype(np.int64) + 32)))


@dataclasses.dataclass
class Samples:
    """Sample pattern caches plus per-pixel choices (aqh_samples)."""
    npatterns: int
    pos: np.ndarray                      # float32[npat, spp, 2]
    time: Optional[np.ndarray] = None    # float32[npat, spp]
    dof: Optional[np.ndarray] = None     # float32[npat, spp, 2]
    shuffle: Optional[np.ndarray] = None  # int32[npat, spp]
    lod: Optional[np.ndarray] = None
    pos_index: Optional[np.ndarray] = None   # uint32[npix]
    dof_index: Optional[np.ndarray] = None
    time_index: Optional[np.ndarray] = None
    shuffle_index: Optional[np.ndarray] = None
    lod_index: Optional[np.ndarray] = None
    dither: Optional[np.ndarray] = None      # float32[crop h * crop w]


@dataclasses.dataclass
class Scene:
    frame: Frame
    grids: Grids
    samples: Samples


# ---------------------------------------------------------------------------
# Sample patterns

def stratified_patterns(xs: int, ys: int, npatterns: int, rng: np.random.Generator,
                        with_time: bool = False, with_dof: bool = False) -> dict:
    """The build's own stratified-jittered pattern cache: sample (ix, iy) lies in
    sub-pixel cell (ix, iy); times are stratified over the spp strata with one
    random offset per pattern (multijitter.cpp:176-190 style); lens positions are
    stratified over the xs*ys lens cells; the lens-shuffle table is a random
    permutation per pattern (multijitter.cpp:192-201 style)."""
    spp = xs * ys
    ix = np.tile(np.arange(xs), ys).astype(np.float32)
    iy = np.repeat(np.arange(ys), xs).astype(np.float32)
    jx = rng.random((npatterns, spp), dtype=np.float32)
    jy = rng.random((npatterns, spp), dtype=np.float32)
    pos = np.empty((npatterns, spp, 2), np.float32)
    pos[..., 0] = (ix + jx) * np.float32(1.0 / xs)
    pos[..., 1] = (iy + jy) * np.float32(1.0 / ys)
    np.clip(pos, 0.0, np.nextafter(np.float32(1.0), np.float32(0.0)), out=pos)
    out = {"pos": pos}
    if with_time:
        delta = np.float32(1.0 / spp)
        r = rng.random((npatterns, 1), dtype=np.float32) * delta
        out["time"] = (np.arange(spp, dtype=np.float32)[None, :] * delta + r).astype(np.float32)
    if with_dof:
        lx = rng.random((npatterns, spp), dtype=np.float32)
        ly = rng.random((npatterns, spp), dtype=np.float32)
        dof = np.empty((npatterns, spp, 2), np.float32)
        dof[..., 0] = (ix + lx) * np.float32(1.0 / xs)
        dof[..., 1] = (iy + ly) * np.float32(1.0 / ys)
        np.clip(dof, 0.0, np.nextafter(np.float32(1.0), np.float32(0.0)), out=dof)
        out["dof"] = dof
        out["shuffle"] = np.argsort(rng.random((npatterns, spp)), axis=1).astype(np.int32)
    return out


def make_samples(frame: Frame, rng: np.random.Generator, npatterns: int = 250,
                 explicit: bool = False, dither: bool = False) -> Samples:
    """Pattern caches of `npatterns` entries picked per pixel at random (as the
    reference's sampler does), or one explicit pattern per pixel."""
    x0, y0, w, h = frame.sample_region
    npix = w * h
    mb = frame.shutter[1] != frame.shutter[0]
    pats = stratified_patterns(frame.xsamples, frame.ysamples, npix if explicit else npatterns, rng,
                               with_time=mb, with_dof=frame.use_dof)
    n = npix if explicit else npatterns

    def idx():
        if explicit:
            return None
        return rng.integers(0, n, npix, dtype=np.uint32)

    cx0, cx1, cy0, cy1 = frame.crop_window
    dith = rng.random((cy1 - cy0) * (cx1 - cx0), dtype=np.float32) if dither else None
    return Samples(npatterns=n, pos=pats["pos"], time=pats.get("time"), dof=pats.get("dof"),
                   shuffle=pats.get("shuffle"), pos_index=idx(), time_index=idx() if mb else None,
                   dof_index=idx() if frame.use_dof else None,
                   shuffle_index=idx() if frame.use_dof else None, dither=dith)


# ---------------------------------------------------------------------------
# Grid streams

def _pack(cu, cv, nkeys, flags, P_list_or_arr, Ci, Oi, times=None, tbase=None) -> Grids:
    G = len(cu)
    nv = (cu.astype(np.int64) + 1) * (cv.astype(np.int64) + 1)
    pbase = np.zeros(G, np.int64)
    pbase[1:] = np.cumsum(nv * nkeys)[:-1]
    cbase = np.zeros(G, np.int64)
    cbase[1:] = np.cumsum(nv)[:-1]
    if times is None:
        times = np.zeros(1, np.float32)
        tbase = np.zeros(G, np.int32)
    return Grids(cu=cu.astype(np.int32), cv=cv.astype(np.int32), nkeys=nkeys.astype(np.int32),
                 flags=flags.astype(np.int32), pbase=pbase, cbase=cbase, tbase=tbase.astype(np.int32),
                 times=times.astype(np.float32), P=P_list_or_arr, Ci=Ci, Oi=Oi)


def regular_grids(ngrids: int, width: int, height: int, rng: np.random.Generator, n: int = 16,
                  jitter: float = 0.3, zrange=(1.0, 1000.0), slope: float = 0.01,
                  window: Optional[tuple] = None, opacity=None, motion: Optional[float] = None,
                  smooth: bool = True, origin_margin: float = 0.0) -> Grids:
    """n x n-quad grids in raster space.  Grid origin uniform over `window`
    (default the image); vertex (i, j) = origin + (i, j) + U[-jitter, jitter]^2;
    z = z0 + s*(x - x0), z0 ~ U[zrange], s ~ U[-slope, slope]; Ci ~ U[0,1]^3;
    Oi = 1, or U[opacity]^3 when `opacity` = (lo, hi).  With `motion` = M a
    second key displaces every vertex of a grid by one vector of length U[0, M]
    in a uniform direction (key times 0 and 1)."""
    nv1 = n + 1
    nvert = nv1 * nv1
    wx0, wx1, wy0, wy1 = window if window is not None else (0.0, float(width), 0.0, float(height))
    ox = rng.uniform(wx0 - origin_margin, wx1, ngrids).astype(np.float32)
    oy = rng.uniform(wy0 - origin_margin, wy1, ngrids).astype(np.float32)
    z0 = rng.uniform(zrange[0], zrange[1], ngrids).astype(np.float32)
    s = rng.uniform(-slope, slope, ngrids).astype(np.float32)
    gi = np.tile(np.arange(nv1, dtype=np.float32), nv1)
    gj = np.repeat(np.arange(nv1, dtype=np.float32), nv1)
    nkeys = 2 if motion is not None else 1
    P = np.empty((ngrids, nkeys, nvert, 4), np.float32)
    jx = rng.uniform(-jitter, jitter, (ngrids, nvert)).astype(np.float32)
    jy = rng.uniform(-jitter, jitter, (ngrids, nvert)).astype(np.float32)
    x = ox[:, None] + gi[None, :] + jx
    y = oy[:, None] + gj[None, :] + jy
    P[:, 0, :, 0] = x
    P[:, 0, :, 1] = y
    P[:, 0, :, 2] = z0[:, None] + s[:, None] * (x - ox[:, None])
    P[:, 0, :, 3] = 0.0
    if motion is not None:
        mag = rng.uniform(0.0, motion, ngrids).astype(np.float32)
        ang = rng.uniform(0.0, 2 * np.pi, ngrids)
        dx = (mag * np.cos(ang)).astype(np.float32)
        dy = (mag * np.sin(ang)).astype(np.float32)
        P[:, 1] = P[:, 0]
        P[:, 1, :, 0] += dx[:, None]
        P[:, 1, :, 1] += dy[:, None]
    Ci = np.empty((ngrids, nvert, 4), np.float32)
    Ci[..., :3] = rng.random((ngrids, nvert, 3), dtype=np.float32)
    Ci[..., 3] = 0.0
    Oi = np.ones((ngrids, nvert, 4), np.float32)
    Oi[..., 3] = 0.0
    flags = np.full(ngrids, GRID_SMOOTH if smooth else 0, np.int32)
    if opacity is not None:
        Oi[..., :3] = rng.uniform(opacity[0], opacity[1], (ngrids, nvert, 3)).astype(np.float32)
    else:
        flags |= GRID_OPAQUE
    cu = np.full(ngrids, n, np.int32)
    cv = np.full(ngrids, n, np.int32)
    times = None
    tbase = None
    if motion is not None:
        times = np.tile(np.array([0.0, 1.0], np.float32), ngrids)
        tbase = np.arange(ngrids, dtype=np.int32) * 2
    return _pack(cu, cv, np.full(ngrids, nkeys, np.int32), flags, P.reshape(-1, 4),
                 Ci.reshape(-1, 4), Oi.reshape(-1, 4), times, tbase)


def concat_grids(parts: list) -> Grids:
    """Concatenate grid streams in order."""
    cu = np.concatenate([g.cu for g in parts])
    cv = np.concatenate([g.cv for g in parts])
    nkeys = np.concatenate([g.nkeys for g in parts])
    flags = np.concatenate([g.flags for g in parts])
    P = np.concatenate([g.P for g in parts])
    Ci = np.concatenate([g.Ci for g in parts])
    Oi = np.concatenate([g.Oi for g in parts])
    times = np.concatenate([g.times for g in parts])
    tb, off = [], 0
    for g in parts:
        tb.append(g.tbase + off)
        off += len(g.times)
    return _pack(cu, cv, nkeys, flags, P, Ci, Oi, times, np.concatenate(tb))


def with_aov(scene: Scene, naov: int = 3, seed: int = 0) -> Scene:
    """The scene with `naov` seeded output variables per vertex, U[-1, 1)."""
    rng = np.random.default_rng(seed)
    aov = rng.uniform(-1.0, 1.0, (len(scene.grids.Ci), naov)).astype(np.float32)
    return Scene(scene.frame, dataclasses.replace(scene.grids, aov=aov), scene.samples)


def with_lod(scene: Scene, seed: int = 0) -> Scene:
    """The scene with seeded sample detail levels U[0, 1) and per-grid
    LevelOfDetailBounds: a mix of off (-1 0), the default (0 1) and random
    windows."""
    rng = np.random.default_rng(seed)
    n = np.asarray(scene.samples.pos).reshape(-1, 2).shape[0]
    lod = rng.random(n).astype(np.float32)
    G = scene.grids.ngrids
    kind = rng.integers(0, 3, G)
    lo = rng.uniform(0.0, 0.6, G)
    hi = lo + rng.uniform(0.2, 0.6, G)
    b = np.stack([np.where(kind == 0, -1.0, np.where(kind == 1, 0.0, lo)),
                  np.where(kind == 0, 0.0, np.where(kind == 1, 1.0, hi))], -1).astype(np.float32)
    # detail levels live in a table of the same patterns as the positions
    smp = dataclasses.replace(scene.samples, lod=lod, lod_index=scene.samples.pos_index)
    return Scene(scene.frame, dataclasses.replace(scene.grids, lod=b), smp)


CSG_PRIMITIVE, CSG_UNION, CSG_INTERSECTION, CSG_DIFFERENCE = 0, 1, 2, 3


def with_csg(scene: Scene, seed: int = 0, ntrees: int = 2, frac: float = 0.6) -> Scene:
    """The scene with seeded CSG trees: `ntrees` solids, each an operation
    node over primitives and (sometimes) a nested operation; about `frac` of
    the grids are primitives of a randomly chosen solid, each grid its own
    primitive node.  The grids of a solid are made two-sided and visible
    from both sides by the caller's scene (their culling state is kept)."""
    rng = np.random.default_rng(seed)
    G = scene.grids.ngrids
    types, parents = [], []
    ops = []  # operation nodes that take primitives
    for _ in range(ntrees):
        root = len(types)
        types.append(int(rng.integers(1, 4)))
        parents.append(-1)
        ops.append(root)
        if rng.random() < 0.5:
            sub = len(types)
            types.append(int(rng.integers(1, 4)))
            parents.append(root)
            ops.append(sub)
    node = np.full(G, -1, np.int32)
    for gi in range(G):
        if rng.random() < frac:
            node[gi] = len(types)
            types.append(CSG_PRIMITIVE)
            parents.append(int(ops[rng.integers(0, len(ops))]))
    g = dataclasses.replace(scene.grids, csg_node=node, csg_type=np.array(types, np.int32),
                            csg_parent=np.array(parents, np.int32))
    return Scene(scene.frame, g, scene.samples)


def trim_sets(loops_per_set, seed=0):
    """Seeded trim sets: each set a list of closed polylines (circles of 8-40
    points at random centres and radii in the unit square, some with a
    second loop inside as a hole).  Returns (points, loop_first, set_first)."""
    rng = np.random.default_rng(seed)
    pts, loop_first, set_first = [], [0], [0]
    for nl in loops_per_set:
        for _ in range(nl):
            n = int(rng.integers(8, 41))
            c = rng.uniform(0.2, 0.8, 2)
            r = rng.uniform(0.1, 0.45)
            a = np.sort(rng.uniform(0, 2 * np.pi, n))
            pts.append(np.stack([c[0] + r * np.cos(a), c[1] + r * np.sin(a)], -1))
            loop_first.append(loop_first[-1] + n)
        set_first.append(set_first[-1] + nl)
    P = np.concatenate(pts).astype(np.float32) if pts else np.zeros((0, 2), np.float32)
    return P, np.array(loop_first, np.int32), np.array(set_first, np.int32)


def with_trim(scene: Scene, seed: int = 0, frac: float = 0.7) -> Scene:
    """The scene with seeded trim curves: each grid's vertices get the
    surface parameters (iu / cu, iv / cv); about `frac` of the grids are
    trimmable, using one of four sets (no loops, one loop, two loops, three
    loops), a quarter of them with the "outside" sense."""
    rng = np.random.default_rng(seed)
    g = scene.grids
    G = g.ngrids
    pts, lf, sf = trim_sets([0, 1, 2, 3], seed=seed + 1)
    uv = np.zeros((len(g.Ci), 2), np.float32)
    for gi in range(G):
        cu, cv = int(g.cu[gi]), int(g.cv[gi])
        U, V = np.meshgrid(np.arange(cu + 1) / max(cu, 1), np.arange(cv + 1) / max(cv, 1))
        # a random affine map of the unit square keeps every set in play
        o = rng.uniform(-0.3, 0.3, 2)
        sc = rng.uniform(0.8, 1.5)
        cb = int(g.cbase[gi])
        uv[cb:cb + (cu + 1) * (cv + 1), 0] = (o[0] + sc * U).ravel()
        uv[cb:cb + (cu + 1) * (cv + 1), 1] = (o[1] + sc * V).ravel()
    tset = np.where(rng.random(G) < frac, rng.integers(0, 4, G), -1).astype(np.int32)
    flags = np.array(g.flags, np.int32, copy=True)
    flags[(tset >= 0) & (rng.random(G) < 0.25)] |= GRID_TRIM_OUTSIDE
    g2 = dataclasses.replace(g, flags=flags, trim_set=tset, trim_uv=uv, trim_points=pts, trim_loop_first=lf,
                             trim_set_first=sf)
    return Scene(scene.frame, g2, scene.samples)


def with_culling(scene: Scene, seed: int = 0) -> Scene:
    """The scene with seeded Shade / Split culling on its camera-space grids:
    a geometric normal per P entry (random directions, so about half the
    vertices face away), shading normals on some grids (flipping Ng where
    they disagree), GRID_CULL_BACKFACING on about 60% of the camera grids
    and GRID_CULL_TRANSPARENT with a trailing run of black Oi on about half."""
    rng = np.random.default_rng(seed)
    g = scene.grids
    Ng = rng.normal(size=(len(g.P), 3)).astype(np.float32)
    N = rng.normal(size=(len(g.P), 3)).astype(np.float32)
    flags = np.array(g.flags, np.int32, copy=True)
    Oi = np.array(g.Oi, np.float32, copy=True)
    cam = (flags & GRID_CAMERA) != 0
    flags[cam & (rng.random(g.ngrids) < 0.6)] |= GRID_CULL_BACKFACING
    tr = cam & (rng.random(g.ngrids) < 0.5)
    flags[tr] |= GRID_CULL_TRANSPARENT
    for i in np.nonzero(tr)[0]:
        nv = (int(g.cu[i]) + 1) * (int(g.cv[i]) + 1)
        run = int(rng.integers(0, nv + 1))
        cb = int(g.cbase[i])
        Oi[cb + nv - run:cb + nv, :3] = 0.0
        flags[i] &= ~GRID_OPAQUE
    use_n = rng.random() < 0.5
    g2 = dataclasses.replace(g, flags=flags, Oi=Oi, cull_Ng=Ng, cull_N=N if use_n else None)
    return Scene(scene.frame, g2, scene.samples)


def opaque_stream(width=1920, height=1080, ngrids=200_000, xs=4, ys=4, seed=0xC1,
                  npatterns=250, explicit_samples=False, filt=("gaussian", 2.0, 2.0)) -> Scene:
    """Opaque synthetic stream: 16x16-quad raster grids, Oi = 1, PixelSamples xs ys."""
    rng = np.random.default_rng(seed)
    fr = Frame(width=width, height=height, xsamples=xs, ysamples=ys, filter=filt[0],
               xfilter=filt[1], yfilter=filt[2], q_dither=0.0)
    g = regular_grids(ngrids, width, height, rng)
    return Scene(fr, g, make_samples(fr, rng, npatterns, explicit_samples))


def transparent_stream(width=1920, height=1080, ngrids=16_200, xs=8, ys=8, seed=0xC2,
                       npatterns=250, explicit_samples=False, window_frac=0.5) -> Scene:
    """Transparent stream: grid origins in a centre window (window_frac of each
    image dimension), Oi ~ U[0.1,0.9]^3, catmull-rom 3x3."""
    rng = np.random.default_rng(seed)
    fr = Frame(width=width, height=height, xsamples=xs, ysamples=ys, filter="catmull-rom",
               xfilter=3.0, yfilter=3.0, q_dither=0.0)
    ww, wh = width * window_frac, height * window_frac
    win = ((width - ww) / 2, (width + ww) / 2, (height - wh) / 2, (height + wh) / 2)
    g = regular_grids(ngrids, width, height, rng, window=win, opacity=(0.1, 0.9))
    return Scene(fr, g, make_samples(fr, rng, npatterns, explicit_samples))


def motion_dof_stream(width=1920, height=1080, ngrids=100_000, xs=6, ys=6, seed=0xC3,
                      npatterns=250, explicit_samples=False, motion=20.0, dof=True,
                      fstop=2.8, focal_length=0.05, focal_distance=50.0,
                      dof_scale=(540.0, 540.0)) -> Scene:
    """Motion blur + depth of field: two keys per vertex with a per-grid
    displacement of length U[0, motion] px; Shutter 0 1; DepthOfField fstop,
    focal length, focal distance; box 1x1 filter."""
    rng = np.random.default_rng(seed)
    fr = Frame(width=width, height=height, xsamples=xs, ysamples=ys, filter="box",
               xfilter=1.0, yfilter=1.0, q_dither=0.0, shutter=(0.0, 1.0) if motion else (0.0, 0.0))
    if dof:
        fr.fstop, fr.focal_length, fr.focal_distance = fstop, focal_length, focal_distance
        fr.dof_scale = dof_scale
    g = regular_grids(ngrids, width, height, rng, motion=motion)
    return Scene(fr, g, make_samples(fr, rng, npatterns, explicit_samples))


def scaled(scene_fn, scale: float, **kw) -> Scene:
    """A smaller copy of a benchmark stream: image and grid count scaled so the
    depth complexity stays the same."""
    w = max(16, int(round(kw.pop("width", 1920) * scale)))
    h = max(16, int(round(kw.pop("height", 1080) * scale)))
    n = kw.pop("ngrids", None)
    if n is None:
        n = {"opaque_stream": 200_000, "transparent_stream": 16_200, "motion_dof_stream": 100_000}[scene_fn.__name__]
    n = max(1, int(round(n * scale * scale)))
    return scene_fn(width=w, height=h, ngrids=n, **kw)


# ---------------------------------------------------------------------------
# Served request stream

SERVED_RESOLUTIONS = [(320, 240), (640, 480), (1280, 720), (1920, 1080), (3840, 2160)]


def served_job(rng: np.random.Generator, seed: int, max_mps: float = 8e6, kind: Optional[str] = None) -> Scene:
    """One request of the served mixed stream: resolution from the five sizes,
    PixelSamples n n with n in {2, 4, 8}, micropolygons log-uniform in
    [50k, 8M] (16x16-quad grids), 20% motion blur + depth of field (two keys,
    displacement U[0,20] px), 30% transparency (Oi ~ U[0.1,0.9]^3, centre
    window), the rest opaque; filters as the stream's base configurations.
    `kind` ("mb", "transparent", "opaque") fixes the request's kind."""
    w, h = SERVED_RESOLUTIONS[int(rng.integers(0, len(SERVED_RESOLUTIONS)))]
    n = int(rng.choice([2, 4, 8]))
    mps = float(np.exp(rng.uniform(np.log(5e4), np.log(max_mps))))
    ngrids = max(1, int(mps / 256))
    k = rng.choice(["mb", "transparent", "opaque"], p=[0.2, 0.3, 0.5])
    kind = k if kind is None else kind
    sub = np.random.default_rng(seed)
    if kind == "mb":
        fr = Frame(width=w, height=h, xsamples=n, ysamples=n, filter="box", xfilter=1.0, yfilter=1.0,
                   q_dither=0.0, shutter=(0.0, 1.0), fstop=2.8, focal_length=0.05, focal_distance=50.0,
                   dof_scale=(h / 2.0, h / 2.0))
        g = regular_grids(ngrids, w, h, sub, motion=20.0)
    elif kind == "transparent":
        fr = Frame(width=w, height=h, xsamples=n, ysamples=n, filter="catmull-rom", xfilter=3.0, yfilter=3.0,
                   q_dither=0.0)
        win = (w * 0.25, w * 0.75, h * 0.25, h * 0.75)
        g = regular_grids(ngrids, w, h, sub, window=win, opacity=(0.1, 0.9))
    else:
        fr = Frame(width=w, height=h, xsamples=n, ysamples=n, q_dither=0.0)
        g = regular_grids(ngrids, w, h, sub)
    sc = Scene(fr, g, make_samples(fr, sub, 250))
    sc.kind = str(kind)
    return sc


def served_stream(njobs: int, seed: int = 0xC4, max_mps: float = 8e6) -> list:
    """`njobs` distinct requests of the served mixed stream with the kinds in
    the configured proportions exactly (20% motion blur + depth of field, 30%
    transparency, the rest opaque; rounded), in a seeded random order."""
    rng = np.random.default_rng(seed)
    nmb = int(round(0.2 * njobs))
    ntr = int(round(0.3 * njobs))
    kinds = ["mb"] * nmb + ["transparent"] * ntr + ["opaque"] * (njobs - nmb - ntr)
    rng.shuffle(kinds)
    return [served_job(rng, 1000 + i, max_mps=max_mps, kind=kinds[i]) for i in range(njobs)]


# ---------------------------------------------------------------------------
# Camera-space grids (the input of Split's projection, AQH_GRID_CAMERA)

def camera_to_raster(width: int, height: int, fov_deg: float = 40.0, near: float = 0.1, far: float = 1e4,
                     orthographic: bool = False, ortho_half_height: float = 100.0) -> tuple:
    """A camera-to-raster matrix as RiProjection "perspective" (or
    "orthographic") followed by the screen-to-raster mapping builds it, in
    CqMatrix element order m[row*4 + col] with points as row vectors.
    Screen window: [-aspect, aspect] x [-1, 1] (scaled by ortho_half_height
    for orthographic), raster y down."""
    aspect = width / height
    l, r, b, t = -aspect, aspect, -1.0, 1.0
    m = np.zeros((4, 4), np.float64)
    if orthographic:
        l, r, b, t = (v * ortho_half_height for v in (l, r, b, t))
        m[0, 0] = width / (r - l)
        m[3, 0] = -l * width / (r - l)
        m[1, 1] = -height / (t - b)
        m[3, 1] = t * height / (t - b)
        m[2, 2] = 1.0 / (far - near)
        m[3, 2] = -near / (far - near)
        m[3, 3] = 1.0
    else:
        f = 1.0 / math.tan(math.radians(fov_deg) / 2)
        m[0, 0] = f * width / (r - l)
        m[2, 0] = -l * width / (r - l)
        m[1, 1] = -f * height / (t - b)
        m[2, 1] = t * height / (t - b)
        m[2, 2] = far / (far - near)
        m[3, 2] = -near * far / (far - near)
        m[2, 3] = 1.0
    return tuple(float(v) for v in m.astype(np.float32).reshape(16))


def to_camera_space(scene: Scene, m=None, every: int = 1, **camera_kw) -> Scene:
    """Turn every `every`-th grid of a raster-space scene into a camera-space
    grid flagged GRID_CAMERA (P unprojected through `m`, float64, then stored
    as float32; camera z unchanged) and set the frame's matrix.  Split's
    projection brings the points back to within rounding of where they were."""
    fr, g = scene.frame, scene.grids
    if m is None:
        m = camera_to_raster(fr.width, fr.height, **camera_kw)
    M = np.asarray(m, np.float64).reshape(4, 4)
    P = np.array(g.P, np.float32, copy=True)
    flags = np.asarray(g.flags, np.int32).copy()
    for i in range(0, g.ngrids, every):
        nv = (int(g.cu[i]) + 1) * (int(g.cv[i]) + 1) * int(g.nkeys[i])
        b = int(g.pbase[i])
        q = P[b:b + nv].astype(np.float64)
        xr, yr, z = q[:, 0], q[:, 1], q[:, 2]
        # h = z m23 + m33; x_r h = x m00 + z m20 + m30 (no x-y coupling in these matrices)
        h = z * M[2, 3] + M[3, 3]
        x = (xr * h - z * M[2, 0] - M[3, 0]) / M[0, 0]
        y = (yr * h - z * M[2, 1] - M[3, 1]) / M[1, 1]
        P[b:b + nv, 0] = x.astype(np.float32)
        P[b:b + nv, 1] = y.astype(np.float32)
        flags[i] |= GRID_CAMERA
    g2 = dataclasses.replace(g, P=P, flags=flags)
    fr2 = dataclasses.replace(fr, camera_to_raster=tuple(float(v) for v in np.asarray(m, np.float32)))
    sc = Scene(fr2, g2, scene.samples)
    if hasattr(scene, "kind"):
        sc.kind = scene.kind
    return sc


# ---------------------------------------------------------------------------
# Scene files

_GRID_KEYS = ("cu", "cv", "nkeys", "flags", "pbase", "cbase", "tbase", "times", "P", "Ci", "Oi", "culled", "aov",
              "lod", "csg_node", "csg_type", "csg_parent", "trim_set", "trim_uv", "trim_points", "trim_loop_first",
              "trim_set_first", "cull_Ng", "cull_N")
_SAMPLE_KEYS = ("pos", "time", "dof", "shuffle", "lod", "pos_index", "dof_index", "time_index",
                "shuffle_index", "lod_index", "dither")


def scene_arrays(scene: Scene) -> dict:
    """Flatten a Scene into named arrays (frame options as a JSON string)."""
    import json
    out = {"frame": np.array(json.dumps(dataclasses.asdict(scene.frame)))}
    for k in _GRID_KEYS:
        a = getattr(scene.grids, k)
        if a is not None:
            out["g_" + k] = np.asarray(a)
    out["s_npatterns"] = np.array(scene.samples.npatterns, np.int64)
    for k in _SAMPLE_KEYS:
        a = getattr(scene.samples, k)
        if a is not None:
            out["s_" + k] = np.asarray(a)
    return out


def scene_from_arrays(d) -> Scene:
    """Inverse of scene_arrays (accepts an NpzFile or a dict)."""
    import json
    fd = json.loads(str(d["frame"]))
    for k in ("crop", "bucket", "shutter", "dof_scale", "zthreshold", "camera_to_raster"):
        if fd.get(k) is not None:
            fd[k] = tuple(fd[k])
    fr = Frame(**fd)
    keys = set(d.keys()) if hasattr(d, "keys") else set(d.files)
    g = Grids(**{k: (np.array(d["g_" + k]) if ("g_" + k) in keys else None) for k in _GRID_KEYS})
    s = Samples(npatterns=int(d["s_npatterns"]),
                **{k: (np.array(d["s_" + k]) if ("s_" + k) in keys else None) for k in _SAMPLE_KEYS})
    return Scene(fr, g, s)


def save_scene(path: str, scene: Scene, **extra) -> None:
    """Write a Scene (plus any extra named arrays) to a compressed .npz file."""
    np.savez_compressed(path, **scene_arrays(scene), **extra)


def load_scene(path: str):
    """Read a Scene written by save_scene; returns (scene, extra arrays)."""
    with np.load(path, allow_pickle=False) as d:
        sc = scene_from_arrays(d)
        extra = {k: np.array(d[k]) for k in d.files if k == "frame" or not (k.startswith("g_") or k.startswith("s_"))}
    extra.pop("frame", None)
    return sc, extra
