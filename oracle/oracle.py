"""ctypes front end of the CPU oracle (oracle/aqh_oracle.cpp).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's
cpu_baseline leg use it as the checker.  Product code never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libaqh_oracle.so")

_f32p = C.POINTER(C.c_float)
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_u32p = C.POINTER(C.c_uint32)
_u8p = C.POINTER(C.c_uint8)
_f64p = C.POINTER(C.c_double)


class OrcFrame(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32),
                ("crop_xmin", C.c_int32), ("crop_xmax", C.c_int32),
                ("crop_ymin", C.c_int32), ("crop_ymax", C.c_int32),
                ("xsamples", C.c_int32), ("ysamples", C.c_int32),
                ("xfilter", C.c_float), ("yfilter", C.c_float),
                ("gain", C.c_float), ("gamma", C.c_float),
                ("q_zero", C.c_float), ("q_one", C.c_float), ("q_min", C.c_float),
                ("q_max", C.c_float), ("q_dither", C.c_float),
                ("shutter_open", C.c_float), ("shutter_close", C.c_float),
                ("use_dof", C.c_int32), ("dof_mult", C.c_float), ("dof_inv_fd", C.c_float),
                ("dof_scale_x", C.c_float), ("dof_scale_y", C.c_float),
                ("depth_filter", C.c_int32), ("zthreshold", C.c_float * 3),
                ("display_z", C.c_int32)]


class OrcGrids(C.Structure):
    _fields_ = [("ngrids", C.c_int32), ("cu", _i32p), ("cv", _i32p), ("nkeys", _i32p),
                ("pbase", _i64p), ("cbase", _i64p), ("tbase", _i64p), ("times", _f32p),
                ("P", _f32p), ("Ci", _f32p), ("Oi", _f32p), ("flags", _i32p), ("culled", _u8p),
                ("aov", _f32p), ("naov", C.c_int32), ("lod", _f32p),
                ("csg_node", _i32p), ("csg_nnodes", C.c_int32), ("csg_type", _i32p), ("csg_parent", _i32p),
                ("trim_set", _i32p), ("trim_uv", _f32p), ("trim_points", _f32p), ("trim_loop_first", _i32p),
                ("trim_set_first", _i32p)]


class OrcSamples(C.Structure):
    _fields_ = [("x0", C.c_int32), ("y0", C.c_int32), ("w", C.c_int32), ("h", C.c_int32),
                ("npatterns", C.c_int32), ("pos", _f32p), ("time", _f32p), ("dof", _f32p),
                ("shuffle", _i32p), ("lod", _f32p), ("pos_index", _u32p), ("dof_index", _u32p),
                ("time_index", _u32p), ("shuffle_index", _u32p), ("lod_index", _u32p),
                ("dither", _f32p)]


class OrcOut(C.Structure):
    _fields_ = [("winner", _i32p), ("occlz", _f32p), ("nfrag", _i32p), ("valid", _u8p),
                ("sdata", _f32p), ("channels", _f32p), ("quantized", _f64p),
                ("qchannels", _i32p), ("nqchannels", C.c_int32),
                ("spl_count", C.c_int64), ("spl_bound_hits", C.c_int64), ("spl_hits", C.c_int64),
                ("aov_channels", _f32p), ("sdata64", _f64p), ("channels64", _f64p)]


def build(quiet: bool = True) -> str:
    """Compile the oracle with its Makefile (gcc only)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.orc_render.argtypes = [C.POINTER(OrcFrame), C.POINTER(OrcGrids), C.POINTER(OrcSamples), _f32p,
                                 C.POINTER(OrcOut)]
        L.orc_render.restype = C.c_int
        L.orc_filter_table.argtypes = [C.c_int, C.c_float, C.c_float, C.c_int, C.c_int, _f32p, C.c_int]
        L.orc_filter_table.restype = C.c_int
        L.orc_filter_eval.argtypes = [C.c_int, C.c_float, C.c_float, C.c_float, C.c_float]
        L.orc_filter_eval.restype = C.c_float
        L.orc_invbilinear.argtypes = [_f32p, _f32p, C.c_int, _f32p]
        L.orc_bilerp2.argtypes = [_f32p, _f32p, C.c_int, _f32p]
        L.orc_mt_seed.argtypes = [C.c_uint32]
        L.orc_mt_int32.restype = C.c_uint32
        L.orc_mt_float.restype = C.c_float
        L.orc_multijitter_tables.argtypes = [C.c_int, C.c_int, _f32p, _f32p, _i32p]
        L.orc_lfloor.argtypes = [C.c_float]
        L.orc_lfloor.restype = C.c_long
        L.orc_lceil.argtypes = [C.c_float]
        L.orc_lceil.restype = C.c_long
        L.orc_project_points.argtypes = [_f32p, _f32p, C.c_int64, _f32p]
        L.orc_cull_grid.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_int, _u8p]
        L.orc_lround.argtypes = [C.c_double]
        L.orc_lround.restype = C.c_long
        L.orc_mag2.argtypes = [C.c_float, C.c_float]
        L.orc_mag2.restype = C.c_float
        L.orc_mag.argtypes = [C.c_float, C.c_float]
        L.orc_mag.restype = C.c_float
        _lib = L
    return _lib


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


def filter_table(filter_id: int, xw: float, yw: float, xs: int, ys: int) -> np.ndarray:
    buf = np.zeros(1 << 16, np.float32)
    n = lib().orc_filter_table(filter_id, xw, yw, xs, ys, _p(buf, _f32p), buf.size)
    if n < 0:
        raise ValueError("filter table too large")
    return buf[:n].copy()


def invbilinear(quad, pts) -> np.ndarray:
    q = np.ascontiguousarray(quad, np.float32).reshape(8)
    P = np.ascontiguousarray(pts, np.float32).reshape(-1, 2)
    uv = np.zeros_like(P)
    lib().orc_invbilinear(_p(q, _f32p), _p(P, _f32p), P.shape[0], _p(uv, _f32p))
    return uv


def bilerp2(quad, uv) -> np.ndarray:
    q = np.ascontiguousarray(quad, np.float32).reshape(8)
    U = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
    P = np.zeros_like(U)
    lib().orc_bilerp2(_p(q, _f32p), _p(U, _f32p), U.shape[0], _p(P, _f32p))
    return P


def multijitter_tables(xs: int, ys: int, seed: int = 545):
    """The reference's 250-entry multi-jitter caches after Reseed(seed)."""
    spp = xs * ys
    pos = np.zeros((250, spp, 2), np.float32)
    t = np.zeros((250, spp), np.float32)
    sh = np.zeros((250, spp), np.int32)
    L = lib()
    L.orc_mt_seed(seed)
    L.orc_multijitter_tables(xs, ys, _p(pos, _f32p), _p(t, _f32p), _p(sh, _i32p))
    return pos, t, sh


def project_points(m, P) -> np.ndarray:
    """Split's camera-to-raster projection (orc_project_points) of float4 points."""
    L = lib()
    m = np.ascontiguousarray(np.asarray(m, np.float32).reshape(16))
    Pin = np.ascontiguousarray(P, np.float32).reshape(-1, 4)
    out = np.empty_like(Pin)
    L.orc_project_points(_p(m, _f32p), _p(Pin, _f32p), Pin.shape[0], _p(out, _f32p))
    return out


def projected_grids(scene):
    """The scene's grids with every GRID_CAMERA grid's keys projected to
    hybrid raster space, as Split leaves them."""
    from aqsis_gb300.scene import GRID_CAMERA
    import dataclasses
    g, m = scene.grids, scene.frame.camera_to_raster
    if m is None or not (np.asarray(g.flags) & GRID_CAMERA).any():
        return g
    P = np.array(g.P, np.float32, copy=True)
    flags = np.asarray(g.flags)
    if getattr(g, "cull_Ng", None) is not None or (flags & 256).any():
        # Shade / Split culling in camera space, before the projection
        L = lib()
        culled = (np.zeros(g.micropolygons, np.uint8) if g.culled is None
                  else np.array(g.culled, np.uint8, copy=True))
        Ng = None if getattr(g, "cull_Ng", None) is None else np.ascontiguousarray(g.cull_Ng, np.float32)
        N = None if getattr(g, "cull_N", None) is None else np.ascontiguousarray(g.cull_N, np.float32)
        Oi = None if g.Oi is None else np.ascontiguousarray(g.Oi, np.float32)
        zblack = int(all(float(z) == 0.0 for z in scene.frame.zthreshold))
        mpb = 0
        for i in range(g.ngrids):
            cu, cv, nk, f = int(g.cu[i]), int(g.cv[i]), int(g.nkeys[i]), int(flags[i])
            if (f & GRID_CAMERA) and (f & (128 | 256)):
                b, cb = int(g.pbase[i]), int(g.cbase[i])
                out = culled[mpb:mpb + cu * cv]
                L.orc_cull_grid(cu, cv, nk, f, _p(P[b:], _f32p), None if Ng is None else _p(Ng[b:], _f32p),
                                None if N is None else _p(N[b:], _f32p), None if Oi is None else _p(Oi[cb:], _f32p),
                                zblack, out.ctypes.data_as(_u8p))
            mpb += cu * cv
        g = dataclasses.replace(g, culled=culled)
    for i in np.nonzero(np.asarray(g.flags) & GRID_CAMERA)[0]:
        nv = (int(g.cu[i]) + 1) * (int(g.cv[i]) + 1) * int(g.nkeys[i])
        b = int(g.pbase[i])
        P[b:b + nv] = project_points(m, P[b:b + nv])
    return dataclasses.replace(g, P=P, flags=np.asarray(g.flags) & ~GRID_CAMERA)


def frame_struct(fr) -> OrcFrame:
    """The OrcFrame of a scene.Frame."""
    cx0, cx1, cy0, cy1 = fr.crop_window
    mult, inv = fr.dof_terms()
    return OrcFrame(fr.width, fr.height, cx0, cx1, cy0, cy1, fr.xsamples, fr.ysamples,
                    fr.xfilter, fr.yfilter, fr.gain, fr.gamma, 0.0, fr.q_one, fr.q_min, fr.q_max,
                    fr.q_dither, fr.shutter[0], fr.shutter[1], 1 if fr.use_dof else 0, mult, inv,
                    fr.dof_scale[0], fr.dof_scale[1], fr.depth_filter,
                    (C.c_float * 3)(*fr.zthreshold), fr.display_z)


def imager(frame, chan, ci_oi) -> np.ndarray:
    """The imager shader's write-back and ExposeBucket (orc_imager) on channels
    FilterBucket left: returns the new channels."""
    L = lib()
    L.orc_imager.argtypes = [C.POINTER(OrcFrame), _f32p, _f32p, C.c_int64]
    L.orc_imager.restype = None
    out = np.array(chan, np.float32, copy=True, order="C")
    im = np.ascontiguousarray(ci_oi, np.float32)
    n = out.reshape(-1, 9).shape[0]
    assert im.size == n * 6
    fs = frame_struct(frame)
    L.orc_imager(C.byref(fs), _p(out, _f32p), _p(im, _f32p), n)
    return out


def quantize(frame, chan, dither=None, qchannels=(0, 1, 2, 6)) -> np.ndarray:
    """FormatBucketForDisplay's quantize (orc_quantize) of channels `qchannels`."""
    L = lib()
    L.orc_quantize.argtypes = [C.POINTER(OrcFrame), _f32p, C.c_int64, _f32p, _i32p, C.c_int, _f64p]
    L.orc_quantize.restype = None
    ch = np.ascontiguousarray(chan, np.float32)
    n = ch.reshape(-1, 9).shape[0]
    qc = np.array(qchannels, np.int32)
    d = None if dither is None else np.ascontiguousarray(dither, np.float32)
    out = np.zeros(ch.shape[:-1] + (len(qc),), np.float64)
    fs = frame_struct(frame)
    L.orc_quantize(C.byref(fs), _p(ch, _f32p), n, _p(d, _f32p), _p(qc, _i32p), len(qc), _p(out, _f64p))
    return out


def render(scene, qchannels=(0, 1, 2, 6), want_samples: bool = True, want_fp64: bool = False,
           grids=None) -> dict:
    """Run the oracle on a Scene (aqsis_gb300.scene).  Returns numpy arrays.
    `want_fp64` adds the float64 twin of Combine and the filter
    ("sdata64" with `want_samples`, "channels64").  `grids` replaces the
    scene's grids after projection (callers that project once)."""
    from aqsis_gb300.scene import FILTERS
    fr, s = scene.frame, scene.samples
    g = projected_grids(scene) if grids is None else grids
    naov = 0 if getattr(g, "aov", None) is None else int(np.asarray(g.aov).reshape(len(g.Ci), -1).shape[1])
    cx0, cx1, cy0, cy1 = fr.crop_window
    x0, y0, w, h = fr.sample_region
    spp = fr.spp
    of = frame_struct(fr)
    keep = []

    def arr(a, dt):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dt)
        keep.append(a)
        return a

    tb = arr(g.tbase.astype(np.int64), np.int64)
    og = OrcGrids(g.ngrids, _p(arr(g.cu, np.int32), _i32p), _p(arr(g.cv, np.int32), _i32p),
                  _p(arr(g.nkeys, np.int32), _i32p), _p(arr(g.pbase, np.int64), _i64p),
                  _p(arr(g.cbase, np.int64), _i64p), _p(tb, _i64p), _p(arr(g.times, np.float32), _f32p),
                  _p(arr(g.P, np.float32), _f32p), _p(arr(g.Ci, np.float32), _f32p),
                  _p(arr(g.Oi, np.float32), _f32p), _p(arr(g.flags, np.int32), _i32p),
                  _p(arr(g.culled, np.uint8), _u8p), _p(arr(getattr(g, "aov", None), np.float32), _f32p),
                  naov, _p(arr(getattr(g, "lod", None), np.float32), _f32p))
    if getattr(g, "csg_node", None) is not None:
        # grids past the given node list are outside any solid
        cn = np.full(g.ngrids, -1, np.int32)
        given = np.asarray(g.csg_node, np.int32).ravel()[:g.ngrids]
        cn[:given.shape[0]] = given
        og.csg_node = _p(arr(cn, np.int32), _i32p)
        og.csg_nnodes = int(np.asarray(g.csg_type).shape[0])
        og.csg_type = _p(arr(g.csg_type, np.int32), _i32p)
        og.csg_parent = _p(arr(g.csg_parent, np.int32), _i32p)
    if getattr(g, "trim_set", None) is not None:
        ts = np.full(g.ngrids, -1, np.int32)
        given = np.asarray(g.trim_set, np.int32).ravel()[:g.ngrids]
        ts[:given.shape[0]] = given
        og.trim_set = _p(arr(ts, np.int32), _i32p)
        og.trim_uv = _p(arr(g.trim_uv, np.float32), _f32p)
        og.trim_points = _p(arr(np.asarray(g.trim_points, np.float32).reshape(-1, 2), np.float32), _f32p)
        og.trim_loop_first = _p(arr(g.trim_loop_first, np.int32), _i32p)
        og.trim_set_first = _p(arr(g.trim_set_first, np.int32), _i32p)
    os_ = OrcSamples(x0, y0, w, h, s.npatterns, _p(arr(s.pos, np.float32), _f32p),
                     _p(arr(s.time, np.float32), _f32p), _p(arr(s.dof, np.float32), _f32p),
                     _p(arr(s.shuffle, np.int32), _i32p), _p(arr(s.lod, np.float32), _f32p),
                     _p(arr(s.pos_index, np.uint32), _u32p), _p(arr(s.dof_index, np.uint32), _u32p),
                     _p(arr(s.time_index, np.uint32), _u32p), _p(arr(s.shuffle_index, np.uint32), _u32p),
                     _p(arr(s.lod_index, np.uint32), _u32p), _p(arr(s.dither, np.float32), _f32p))
    ftab = filter_table(FILTERS[fr.filter], fr.xfilter, fr.yfilter, fr.xsamples, fr.ysamples)
    ns = w * h * spp
    dw, dh = cx1 - cx0, cy1 - cy0
    res = {}
    if want_samples:
        res["winner"] = np.zeros(ns, np.int32)
        res["occlz"] = np.zeros(ns, np.float32)
        res["nfrag"] = np.zeros(ns, np.int32)
        res["valid"] = np.zeros(ns, np.uint8)
        res["sdata"] = np.zeros((ns, 7), np.float32)
    res["channels"] = np.zeros((dh, dw, 9), np.float32)
    qc = np.array(qchannels, np.int32)
    res["quantized"] = np.zeros((dh, dw, len(qc)), np.float64)
    if naov:
        res["aov"] = np.zeros((dh, dw, naov), np.float32)
    if want_fp64:
        res["channels64"] = np.zeros((dh, dw, 9), np.float64)
        if want_samples:
            res["sdata64"] = np.zeros((ns, 7), np.float64)
    oo = OrcOut(_p(res.get("winner"), _i32p), _p(res.get("occlz"), _f32p), _p(res.get("nfrag"), _i32p),
                _p(res.get("valid"), _u8p), _p(res.get("sdata"), _f32p), _p(res["channels"], _f32p),
                _p(res["quantized"], _f64p), _p(qc, _i32p), len(qc), 0, 0, 0, _p(res.get("aov"), _f32p),
                _p(res.get("sdata64"), _f64p), _p(res.get("channels64"), _f64p))
    rc = lib().orc_render(C.byref(of), C.byref(og), C.byref(os_), _p(ftab, _f32p), C.byref(oo))
    if rc != 0:
        raise RuntimeError("oracle render failed: %d" % rc)
    res["spl_count"], res["spl_bound_hits"], res["spl_hits"] = oo.spl_count, oo.spl_bound_hits, oo.spl_hits
    return res


def strip_scene(scene, y0: int, y1: int):
    """The scene restricted to display rows [y0, y1) of its crop window: the
    same grids, a crop window of those rows, and the sample choices of the
    rows of the full sample region that the strip's sample region covers, so
    that every sample of the strip is the one the whole frame has there."""
    import dataclasses
    fr = scene.frame
    cx0, cx1, cy0, cy1 = fr.crop_window
    assert cy0 <= y0 < y1 <= cy1
    X0, Y0, W, H = fr.sample_region
    f2 = dataclasses.replace(fr, crop=(cx0, cx1, y0, y1))
    x0, sy0, w, h = f2.sample_region
    r0 = sy0 - Y0
    s = scene.samples

    def rows(idx):
        full = np.arange(W * H, dtype=np.uint32) if idx is None else np.asarray(idx, np.uint32)
        return np.ascontiguousarray(full.reshape(H, W)[r0:r0 + h].ravel())

    kw = {"pos_index": rows(s.pos_index)}
    for k in ("time_index", "dof_index", "shuffle_index", "lod_index"):
        src = getattr(s, k)
        if src is not None or getattr(s, k.replace("_index", "")) is not None:
            kw[k] = rows(src)
    if s.dither is not None:
        dw = cx1 - cx0
        kw["dither"] = np.ascontiguousarray(np.asarray(s.dither).reshape(cy1 - cy0, dw)[y0 - cy0:y1 - cy0].ravel())
    return type(scene)(f2, scene.grids, dataclasses.replace(s, **kw))


def render_strips(scene, nthreads: int = 0, qchannels=(0, 1, 2, 6), want_fp64: bool = False,
                  nstrips: int = 0) -> dict:
    """The oracle over a whole frame in horizontal strips, one host thread per
    strip (the oracle keeps no global state, and ctypes drops the GIL while
    it runs).  Channels, quantized values and the float64 twin's channels,
    stitched in display order."""
    from concurrent.futures import ThreadPoolExecutor
    fr = scene.frame
    cx0, cx1, cy0, cy1 = fr.crop_window
    n = nthreads or os.cpu_count() or 1
    k = max(1, min(nstrips or 4 * n, cy1 - cy0))
    g = projected_grids(scene)
    edges = [cy0 + (cy1 - cy0) * i // k for i in range(k + 1)]
    parts = [(edges[i], edges[i + 1]) for i in range(k) if edges[i + 1] > edges[i]]
    ybounds = _grid_ybounds(g) if not fr.use_dof else None

    def one(b):
        gs = g
        if ybounds is not None:
            # grids whose raster y range (every key) reaches the strip's
            # AddMPG window, in their original order: the others are culled
            # by the oracle anyway, and a subset in the same order keeps
            # every sample's sequence of candidates
            m = (ybounds[1] >= b[0] - fr.yfilter / 2.0 - 2.0) & (ybounds[0] <= b[1] + fr.yfilter / 2.0 + 2.0)
            gs = _grid_subset(g, np.nonzero(m)[0])
        return render(strip_scene(scene, *b), qchannels, want_samples=False, want_fp64=want_fp64, grids=gs)

    with ThreadPoolExecutor(max_workers=n) as ex:
        outs = list(ex.map(one, parts))
    res = {key: np.concatenate([o[key] for o in outs], axis=0)
           for key in ("channels", "quantized") + (("channels64",) if want_fp64 else ())}
    return res


def _grid_ybounds(g):
    """Per grid (min, max) raster y over every key, or None when the grids
    are not packed back to back in P (then no strip culling is done) or
    carry per-grid extras that a subset would have to renumber."""
    for k in ("aov", "lod", "csg_node", "trim_set", "culled"):
        if getattr(g, k, None) is not None:
            return None
    nv = (g.cu.astype(np.int64) + 1) * (g.cv.astype(np.int64) + 1) * g.nkeys.astype(np.int64)
    pb = np.asarray(g.pbase, np.int64)
    if g.ngrids == 0 or pb[0] != 0 or not np.array_equal(pb[1:], np.cumsum(nv)[:-1]):
        return None
    y = np.ascontiguousarray(np.asarray(g.P)[:int(nv.sum()), 1])
    return np.minimum.reduceat(y, pb), np.maximum.reduceat(y, pb)


def _grid_subset(g, idx):
    import dataclasses
    return dataclasses.replace(g, cu=g.cu[idx], cv=g.cv[idx], nkeys=g.nkeys[idx], flags=g.flags[idx],
                               pbase=g.pbase[idx], cbase=g.cbase[idx], tbase=g.tbase[idx])


def fp64_error(dev, ref64, finite_only: bool = True) -> dict:
    """Largest absolute and relative difference of float results `dev` from
    the float64 twin `ref64` (relative over entries with |ref64| >= 1e-6).
    Entries where the twin is not finite or at FLT_MAX (an empty pixel's
    depth) are left out, and so are entries where the float result is not
    finite while the twin is (the float sum overflowed, as in the reference's
    own float path, near FLT_MAX depths under negative filter lobes); those
    are counted as `float_overflow`."""
    a = np.asarray(dev, np.float64)
    b = np.asarray(ref64, np.float64)
    tw = np.isfinite(b) & (np.abs(b) < 3.0e38) if finite_only else np.ones(b.shape, bool)
    ovf = tw & ~np.isfinite(a)
    m = tw & np.isfinite(a)
    if not m.any():
        return {"max_abs": 0.0, "max_rel": 0.0, "entries": 0, "float_overflow": int(ovf.sum())}
    d = np.abs(a[m] - b[m])
    big = np.abs(b[m]) >= 1e-6
    rel = float((d[big] / np.abs(b[m][big])).max()) if big.any() else 0.0
    return {"max_abs": float(d.max()), "max_rel": rel, "entries": int(m.sum()), "float_overflow": int(ovf.sum())}
