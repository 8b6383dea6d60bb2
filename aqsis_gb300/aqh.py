"""ctypes front end of libaqh (include/aqh.h), the GB300 hider.

This mirrors the reference's hider boundary for Python callers and tests:
``Hider.frame_begin`` takes the RI frame options, ``submit_grid`` /
``submit_scene`` stand in for CqImageBuffer::AddMPG, ``render`` for
CqImageBuffer::RenderImage, and ``read_channels`` / ``read_bucket`` /
``read_quantized`` hand back what CqDDManager::DisplayBucket receives.

The library must be built (``aqsis_gb300.build.build()``); there is no
fallback -- loading fails loudly when the shared object is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import build as _build
from .scene import FILTERS, Scene

_f32p = C.POINTER(C.c_float)
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_u32p = C.POINTER(C.c_uint32)
_u8p = C.POINTER(C.c_uint8)

AQH_OK = 0
STATUS = {0: "AQH_OK", 1: "AQH_EINVAL", 2: "AQH_ENOMEM", 3: "AQH_EDEVICE", 4: "AQH_ETIMEDOUT",
          5: "AQH_EREJECTED", 6: "AQH_ENOTREADY", 7: "AQH_ELIMIT"}


class AqhError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


class FrameDesc(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int),
                ("crop_xmin", C.c_int), ("crop_xmax", C.c_int), ("crop_ymin", C.c_int), ("crop_ymax", C.c_int),
                ("bucket_x", C.c_int), ("bucket_y", C.c_int),
                ("xsamples", C.c_int), ("ysamples", C.c_int),
                ("xfilter", C.c_float), ("yfilter", C.c_float), ("filter", C.c_int),
                ("gain", C.c_float), ("gamma", C.c_float),
                ("q_one", C.c_float), ("q_min", C.c_float), ("q_max", C.c_float), ("q_dither", C.c_float),
                ("shutter_open", C.c_float), ("shutter_close", C.c_float),
                ("fstop", C.c_float), ("focal_length", C.c_float), ("focal_distance", C.c_float),
                ("dof_scale_x", C.c_float), ("dof_scale_y", C.c_float),
                ("depth_filter", C.c_int), ("zthreshold", C.c_float * 3), ("display_z", C.c_int)]


class Grid(C.Structure):
    _fields_ = [("cu", C.c_int), ("cv", C.c_int), ("nkeys", C.c_int), ("key_times", _f32p),
                ("P", _f32p), ("Ci", _f32p), ("Oi", _f32p), ("culled", _u8p), ("flags", C.c_int),
                ("aov", _f32p)]


class Samples(C.Structure):
    _fields_ = [("npatterns", C.c_int), ("pos", _f32p), ("time", _f32p), ("dof", _f32p), ("shuffle", _i32p),
                ("lod", _f32p), ("pos_index", _u32p), ("dof_index", _u32p), ("time_index", _u32p),
                ("shuffle_index", _u32p), ("lod_index", _u32p), ("dither", _f32p)]


class FrameStats(C.Structure):
    _fields_ = [("micropolygons", C.c_int64), ("samples", C.c_int64), ("grids", C.c_int64),
                ("tile_grid_pairs", C.c_int64), ("fragments", C.c_int64),
                ("ms_bin", C.c_float), ("ms_sample", C.c_float), ("ms_filter", C.c_float), ("ms_total", C.c_float),
                ("graphs_built", C.c_int64), ("rerenders", C.c_int64)]


class Tuning(C.Structure):
    _fields_ = [("tile_pixels", C.c_int), ("supertile_pixels", C.c_int), ("persistent_ctas", C.c_int),
                ("filter_ctas_per_sm", C.c_int), ("ms", C.c_float)]


class Display(C.Structure):
    _fields_ = [("nchan", C.c_int), ("channels", C.c_int * 16), ("q_zero", C.c_float), ("q_one", C.c_float),
                ("q_min", C.c_float), ("q_max", C.c_float), ("q_dither", C.c_float), ("format", C.c_int),
                ("dither", C.c_void_p)]


# AQH_DSPY_* element types (PkDspy* codes) and their numpy dtypes
DSPY_DTYPES = {1: np.float32, 2: np.uint32, 3: np.int32, 4: np.uint16, 5: np.int16, 6: np.uint8, 7: np.int8}


class DspyGeometry(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("origin_x", C.c_int), ("origin_y", C.c_int),
                ("full_width", C.c_int), ("full_height", C.c_int), ("bucket_x", C.c_int), ("bucket_y", C.c_int)]


def capture_driver_path() -> str:
    """The headless display driver built with the library (writes PPM / raw files)."""
    import os
    return os.path.join(os.path.dirname(_build.LIB), "libaqh_dspy_capture.so")


def make_display(channels, one=255.0, qmin=0.0, qmax=255.0, dither_amp=0.5, zero=0.0, fmt=0, dither=None):
    d = Display()
    d.nchan = len(channels)
    for i, c in enumerate(channels):
        d.channels[i] = int(c)
    d.q_zero, d.q_one, d.q_min, d.q_max, d.q_dither = zero, one, qmin, qmax, dither_amp
    d.format = int(fmt)
    keep = None
    if dither is not None:
        keep = np.ascontiguousarray(dither, np.float32).reshape(-1)
        d.dither = keep.ctypes.data
    return d, keep


class DisplayDriver:
    """A Dspy display driver fed by the library (aqh_dspy_open / _send / _close)."""

    def __init__(self, driver: str, filename: str, geometry: DspyGeometry, channels, names, **quantize):
        self.L = load()
        self.d, self._keep = make_display(channels, **quantize)
        arr = (C.c_char_p * len(names))(*[n.encode() for n in names])
        self._names = arr
        self.h = C.c_void_p()
        rc = self.L.aqh_dspy_open(driver.encode(), filename.encode(), C.byref(geometry), C.byref(self.d), arr,
                                  C.byref(self.h))
        if rc != AQH_OK:
            raise AqhError(rc, "aqh_dspy_open: " + self.L.aqh_dspy_last_error().decode())

    def send(self, hider):
        rc = self.L.aqh_dspy_send(self.h, hider.ctx)
        if rc != AQH_OK:
            raise AqhError(rc, "aqh_dspy_send: " + self.L.aqh_dspy_last_error().decode())

    def send_image(self, image: np.ndarray):
        image = np.ascontiguousarray(image)
        rc = self.L.aqh_dspy_send_image(self.h, image.ctypes.data, image.nbytes)
        if rc != AQH_OK:
            raise AqhError(rc, "aqh_dspy_send_image: " + self.L.aqh_dspy_last_error().decode())

    def close(self):
        if self.h:
            rc = self.L.aqh_dspy_close(self.h)
            self.h = C.c_void_p()
            if rc != AQH_OK:
                raise AqhError(rc, "aqh_dspy_close: " + self.L.aqh_dspy_last_error().decode())


class DeviceOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("vertex_capacity", C.c_size_t), ("grid_capacity", C.c_size_t)]


_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load libaqh.so.  Raises if it is missing (no fallback path exists)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError("libaqh.so is not built (%s); run aqsis_gb300.build.build()" % path)
    L = C.CDLL(path)
    vp = C.c_void_p
    L.aqh_create.argtypes = [C.POINTER(DeviceOpts), C.POINTER(vp)]
    L.aqh_destroy.argtypes = [vp]
    L.aqh_destroy.restype = None
    L.aqh_last_error.argtypes = [vp]
    L.aqh_last_error.restype = C.c_char_p
    L.aqh_status_string.argtypes = [C.c_int]
    L.aqh_status_string.restype = C.c_char_p
    L.aqh_frame_desc_defaults.argtypes = [C.POINTER(FrameDesc)]
    L.aqh_frame_desc_defaults.restype = None
    L.aqh_frame_begin.argtypes = [vp, C.POINTER(FrameDesc)]
    L.aqh_set_imager.argtypes = [vp, C.c_int]
    L.aqh_apply_imager.argtypes = [vp, _f32p, C.c_size_t]
    L.aqh_set_samples.argtypes = [vp, C.POINTER(Samples)]
    L.aqh_submit_grid.argtypes = [vp, C.POINTER(Grid)]
    L.aqh_submit_grids_device.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, C.c_int64]
    L.aqh_render.argtypes = [vp, C.c_int]
    L.aqh_set_mode.argtypes = [vp, C.c_int]
    L.aqh_set_stream.argtypes = [vp, vp]
    L.aqh_synchronize.argtypes = [vp]
    L.aqh_read_channels.argtypes = [vp, _f32p, C.c_size_t]
    L.aqh_read_bucket.argtypes = [vp, C.c_int, C.c_int, _f32p, C.c_size_t, _i32p, _i32p]
    L.aqh_read_quantized_u8.argtypes = [vp, _i32p, C.c_int, _u8p, C.c_size_t]
    L.aqh_read_samples.argtypes = [vp, _i32p, _f32p, _i32p, _u8p, _f32p, C.c_size_t]
    L.aqh_get_stats.argtypes = [vp, C.POINTER(FrameStats)]
    L.aqh_set_camera_to_raster.argtypes = [vp, _f32p]
    L.aqh_set_aov_count.argtypes = [vp, C.c_int]
    L.aqh_set_lod_bounds.argtypes = [vp, _f32p, C.c_int]
    L.aqh_set_csg.argtypes = [vp, _i32p, _i32p, C.c_int, _i32p, C.c_int]
    L.aqh_set_host_copy.argtypes = [vp, C.c_int]
    L.aqh_set_cull_normals.argtypes = [vp, _f32p, _f32p, C.c_size_t]
    L.aqh_set_trim.argtypes = [vp, _i32p, C.c_int, _f32p, C.c_size_t, _f32p, C.c_int, _i32p, C.c_int, _i32p, C.c_int]
    L.aqh_dspy_geometry_of.argtypes = [vp, C.POINTER(DspyGeometry)]
    L.aqh_dspy_open.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(DspyGeometry), C.POINTER(Display),
                                C.POINTER(C.c_char_p), C.POINTER(vp)]
    L.aqh_dspy_send.argtypes = [vp, vp]
    L.aqh_dspy_send_image.argtypes = [vp, vp, C.c_size_t]
    L.aqh_dspy_close.argtypes = [vp]
    L.aqh_dspy_last_error.restype = C.c_char_p
    L.aqh_submit_aov_host.argtypes = [vp, _f32p, C.c_size_t]
    L.aqh_submit_aov_device.argtypes = [vp, vp]
    L.aqh_read_aov.argtypes = [vp, _f32p, C.c_size_t]
    L.aqh_display_format.argtypes = [C.c_float, C.c_float, C.c_float]
    L.aqh_display_format.restype = C.c_int
    L.aqh_read_display.argtypes = [vp, C.POINTER(Display), vp, C.c_size_t, C.POINTER(C.c_int)]
    L.aqh_set_tuning.argtypes = [vp, C.POINTER(Tuning)]
    L.aqh_get_tuning.argtypes = [vp, C.POINTER(Tuning)]
    L.aqh_autotune.argtypes = [vp, C.c_int, C.POINTER(Tuning)]
    L.aqh_filter_table.argtypes = [C.c_int, C.c_float, C.c_float, C.c_int, C.c_int, _f32p, C.c_int]
    L.aqh_filter_table.restype = C.c_int
    L.aqh_test_invbilinear.argtypes = [_f32p, _f32p, C.c_int, _f32p]
    for name in ("aqh_create", "aqh_set_mode", "aqh_set_stream", "aqh_frame_begin", "aqh_set_samples", "aqh_submit_grid", "aqh_submit_grids_device",
                 "aqh_render", "aqh_synchronize", "aqh_read_channels", "aqh_read_bucket", "aqh_read_quantized_u8",
                 "aqh_read_samples", "aqh_get_stats", "aqh_test_invbilinear", "aqh_set_tuning", "aqh_get_tuning",
                 "aqh_autotune", "aqh_set_camera_to_raster", "aqh_read_display", "aqh_set_aov_count",
                 "aqh_submit_aov_host", "aqh_submit_aov_device", "aqh_read_aov", "aqh_dspy_geometry_of",
                 "aqh_dspy_open", "aqh_dspy_send", "aqh_dspy_send_image", "aqh_dspy_close", "aqh_set_lod_bounds",
                 "aqh_set_csg", "aqh_set_trim", "aqh_set_host_copy",
                 "aqh_set_cull_normals"):
        getattr(L, name).restype = C.c_int
    _lib = L
    return L


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


def frame_desc(fr) -> FrameDesc:
    """aqh_frame_desc from an aqsis_gb300.scene.Frame."""
    d = FrameDesc()
    load().aqh_frame_desc_defaults(C.byref(d))
    d.width, d.height = fr.width, fr.height
    if fr.crop is not None:
        d.crop_xmin, d.crop_xmax, d.crop_ymin, d.crop_ymax = fr.crop
    d.bucket_x, d.bucket_y = fr.bucket
    d.xsamples, d.ysamples = fr.xsamples, fr.ysamples
    d.xfilter, d.yfilter = fr.xfilter, fr.yfilter
    d.filter = FILTERS[fr.filter]
    d.gain, d.gamma = fr.gain, fr.gamma
    d.q_one, d.q_min, d.q_max, d.q_dither = fr.q_one, fr.q_min, fr.q_max, fr.q_dither
    d.shutter_open, d.shutter_close = fr.shutter
    d.fstop, d.focal_length, d.focal_distance = fr.fstop, fr.focal_length, fr.focal_distance
    d.dof_scale_x, d.dof_scale_y = fr.dof_scale
    d.depth_filter = fr.depth_filter
    d.zthreshold = (C.c_float * 3)(*fr.zthreshold)
    d.display_z = fr.display_z
    return d


def filter_table(filter_id: int, xw: float, yw: float, xs: int, ys: int) -> np.ndarray:
    L = load()
    n = -L.aqh_filter_table(filter_id, xw, yw, xs, ys, None, 0)
    out = np.zeros(max(n, 1), np.float32)
    L.aqh_filter_table(filter_id, xw, yw, xs, ys, _p(out, _f32p), n)
    return out[:n]


def invbilinear(quad, pts) -> np.ndarray:
    """Device CqInvBilinear lookups (test hook)."""
    q = np.ascontiguousarray(quad, np.float32).reshape(8)
    P = np.ascontiguousarray(pts, np.float32).reshape(-1, 2)
    uv = np.zeros_like(P)
    rc = load().aqh_test_invbilinear(_p(q, _f32p), _p(P, _f32p), P.shape[0], _p(uv, _f32p))
    if rc != AQH_OK:
        raise AqhError(rc, "aqh_test_invbilinear failed")
    return uv


class Hider:
    """One hider context (aqh_ctx) on one CUDA device."""

    def __init__(self, device: int = 0):
        self.L = load()
        self.ctx = C.c_void_p()
        opts = DeviceOpts(device, 0, 0)
        self._check(self.L.aqh_create(C.byref(opts), C.byref(self.ctx)), "aqh_create")
        self._keep = []
        self.frame = None

    def close(self):
        if self.ctx:
            self.L.aqh_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int, what: str):
        if rc != AQH_OK:
            msg = self.L.aqh_last_error(self.ctx).decode() if self.ctx else what
            raise AqhError(rc, "%s: %s" % (what, msg))

    # ---- frame --------------------------------------------------------------
    def frame_begin(self, fr):
        self.frame = fr
        self._keep = []
        self.naov = 0
        self._check(self.L.aqh_frame_begin(self.ctx, C.byref(frame_desc(fr))), "aqh_frame_begin")
        if getattr(fr, "camera_to_raster", None) is not None:
            self.set_camera_to_raster(fr.camera_to_raster)

    def set_camera_to_raster(self, m):
        """Camera-to-raster matrix (16 floats, m[row*4 + col]) for GRID_CAMERA
        grids (aqh_set_camera_to_raster); None clears it."""
        if m is None:
            self._check(self.L.aqh_set_camera_to_raster(self.ctx, None), "aqh_set_camera_to_raster")
            return
        a = np.ascontiguousarray(np.asarray(m, np.float32).reshape(16))
        self._check(self.L.aqh_set_camera_to_raster(self.ctx, _p(a, _f32p)), "aqh_set_camera_to_raster")

    def set_samples(self, s):
        keep = []

        def a(x, dt):
            if x is None:
                return None
            x = np.ascontiguousarray(x, dt)
            keep.append(x)
            return x
        cs = Samples(int(s.npatterns), _p(a(s.pos, np.float32), _f32p), _p(a(s.time, np.float32), _f32p),
                     _p(a(s.dof, np.float32), _f32p), _p(a(s.shuffle, np.int32), _i32p),
                     _p(a(s.lod, np.float32), _f32p), _p(a(s.pos_index, np.uint32), _u32p),
                     _p(a(s.dof_index, np.uint32), _u32p), _p(a(s.time_index, np.uint32), _u32p),
                     _p(a(s.shuffle_index, np.uint32), _u32p), _p(a(s.lod_index, np.uint32), _u32p),
                     _p(a(s.dither, np.float32), _f32p))
        self._check(self.L.aqh_set_samples(self.ctx, C.byref(cs)), "aqh_set_samples")
        self._check(self.L.aqh_synchronize(self.ctx), "aqh_synchronize")

    def set_lod_bounds(self, bounds):
        """LevelOfDetailBounds per grid, float[G][2] (aqh_set_lod_bounds)."""
        b = np.ascontiguousarray(bounds, np.float32).reshape(-1, 2)
        self._check(self.L.aqh_set_lod_bounds(self.ctx, _p(b, _f32p), b.shape[0]), "aqh_set_lod_bounds")

    def set_csg(self, node_type, node_parent, grid_node):
        """The frame's CSG trees and each grid's primitive node (aqh_set_csg)."""
        t = np.ascontiguousarray(node_type, np.int32).ravel()
        par = np.ascontiguousarray(node_parent, np.int32).ravel()
        gn = np.ascontiguousarray(grid_node, np.int32).ravel()
        if t.shape != par.shape:
            raise ValueError("node_type and node_parent differ in length")
        self._check(self.L.aqh_set_csg(self.ctx, _p(t, _i32p), _p(par, _i32p), t.shape[0], _p(gn, _i32p),
                                       gn.shape[0]), "aqh_set_csg")

    def set_trim(self, grid_set, uv, points, loop_first, set_first):
        """Trim curves (aqh_set_trim): each grid's trim set, per-vertex (u, v)
        indexed like Ci, and the sets as loops of points."""
        gs = np.ascontiguousarray(grid_set, np.int32).ravel()
        uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 2)
        lf = np.ascontiguousarray(loop_first, np.int32).ravel()
        sf = np.ascontiguousarray(set_first, np.int32).ravel()
        self._check(self.L.aqh_set_trim(self.ctx, _p(gs, _i32p), gs.shape[0], _p(uv, _f32p), uv.shape[0],
                                        _p(pts, _f32p), pts.shape[0], _p(lf, _i32p), lf.shape[0] - 1,
                                        _p(sf, _i32p), sf.shape[0] - 1), "aqh_set_trim")

    def set_aov_count(self, n: int):
        """Output variables per vertex for this frame (aqh_set_aov_count), before any grid."""
        self._check(self.L.aqh_set_aov_count(self.ctx, int(n)), "aqh_set_aov_count")
        self.naov = int(n)

    def read_aov(self) -> np.ndarray:
        w, h = self._dims()
        out = np.zeros((h, w, self.naov), np.float32)
        self._check(self.L.aqh_read_aov(self.ctx, _p(out, _f32p), out.size), "aqh_read_aov")
        return out

    def submit_grid(self, cu, cv, P, Ci=None, Oi=None, flags=1, key_times=None, culled=None, aov=None):
        P = np.ascontiguousarray(P, np.float32)
        nkeys = 1 if key_times is None else len(key_times)
        kt = None if key_times is None else np.ascontiguousarray(key_times, np.float32)
        Ci = None if Ci is None else np.ascontiguousarray(Ci, np.float32)
        Oi = None if Oi is None else np.ascontiguousarray(Oi, np.float32)
        cl = None if culled is None else np.ascontiguousarray(culled, np.uint8)
        av = None if aov is None else np.ascontiguousarray(aov, np.float32)
        g = Grid(cu, cv, nkeys, _p(kt, _f32p), _p(P, _f32p), _p(Ci, _f32p), _p(Oi, _f32p), _p(cl, _u8p), flags,
                 _p(av, _f32p))
        self._check(self.L.aqh_submit_grid(self.ctx, C.byref(g)), "aqh_submit_grid")

    def submit_scene_grids(self, g):
        """Submit every grid of a scene.Grids through aqh_submit_grid, in order."""
        mpbase = 0
        aov = None
        if getattr(g, "aov", None) is not None:
            aov = np.asarray(g.aov, np.float32).reshape(len(g.Ci), -1)
            self.set_aov_count(aov.shape[1])
        for i in range(g.ngrids):
            cu, cv, nk = int(g.cu[i]), int(g.cv[i]), int(g.nkeys[i])
            nv = (cu + 1) * (cv + 1)
            pb, cb = int(g.pbase[i]), int(g.cbase[i])
            kt = None
            if nk > 1:
                kt = g.times[int(g.tbase[i]):int(g.tbase[i]) + nk]
            cl = None
            if g.culled is not None:
                cl = g.culled[mpbase:mpbase + cu * cv]
            self.submit_grid(cu, cv, g.P[pb:pb + nv * nk], g.Ci[cb:cb + nv], g.Oi[cb:cb + nv], int(g.flags[i]),
                             kt, cl, None if aov is None else aov[cb:cb + nv])
            mpbase += cu * cv
        if getattr(g, "lod", None) is not None:
            self.set_lod_bounds(g.lod)
        if getattr(g, "csg_node", None) is not None:
            self.set_csg(g.csg_type, g.csg_parent, g.csg_node)
        if getattr(g, "trim_set", None) is not None:
            self.set_trim(g.trim_set, g.trim_uv, g.trim_points, g.trim_loop_first, g.trim_set_first)
        if getattr(g, "cull_Ng", None) is not None or (np.asarray(g.flags) & 256).any():
            self.set_cull_normals(getattr(g, "cull_Ng", None), getattr(g, "cull_N", None))

    def submit_grids_host(self, g, packed3: bool = False):
        """Submit a whole packed scene.Grids in one aqh_submit_grids_host call
        (the arrays are copied to the device at render time, so they must stay
        alive until then; they are kept on the object).  packed3: P, Ci and Oi
        as three-float entries (aqh_submit_grids_host3)."""
        L = self.L
        if not getattr(L, "_packed_bound", False):
            vp = C.c_void_p
            for fn in (L.aqh_submit_grids_host, L.aqh_submit_grids_host3):
                fn.argtypes = [vp, C.c_int] + [vp] * 8 + [C.c_size_t, vp, C.c_size_t, vp, vp, C.c_size_t, vp,
                                                          C.c_int64]
                fn.restype = C.c_int
            L._packed_bound = True
        keep = []

        def a(x, dt):
            x = np.ascontiguousarray(x, dt)
            keep.append(x)
            return x.ctypes.data
        culled = a(g.culled, np.uint8) if g.culled is not None else None
        av = None
        if getattr(g, "aov", None) is not None:
            av = np.ascontiguousarray(np.asarray(g.aov, np.float32).reshape(len(g.Ci), -1))
            self.set_aov_count(av.shape[1])
        fn = L.aqh_submit_grids_host3 if packed3 else L.aqh_submit_grids_host
        k = 3 if packed3 else 4
        self._check(fn(self.ctx, g.ngrids, a(g.cu, np.int32), a(g.cv, np.int32),
                       a(g.nkeys, np.int32), a(g.flags, np.int32), a(g.pbase, np.int64),
                       a(g.cbase, np.int64), a(g.tbase, np.int32), a(g.times, np.float32),
                       int(g.times.size), a(np.asarray(g.P)[:, :k], np.float32), int(g.P.shape[0]),
                       a(np.asarray(g.Ci)[:, :k], np.float32), a(np.asarray(g.Oi)[:, :k], np.float32),
                       int(g.Ci.shape[0]), culled, g.micropolygons),
                    "aqh_submit_grids_host3" if packed3 else "aqh_submit_grids_host")
        if av is not None:
            self._check(L.aqh_submit_aov_host(self.ctx, _p(av, _f32p), av.shape[0]), "aqh_submit_aov_host")
            keep.append(av)
        if getattr(g, "lod", None) is not None:
            self.set_lod_bounds(g.lod)
        if getattr(g, "csg_node", None) is not None:
            self.set_csg(g.csg_type, g.csg_parent, g.csg_node)
        if getattr(g, "trim_set", None) is not None:
            self.set_trim(g.trim_set, g.trim_uv, g.trim_points, g.trim_loop_first, g.trim_set_first)
        if getattr(g, "cull_Ng", None) is not None or (np.asarray(g.flags) & 256).any():
            self.set_cull_normals(getattr(g, "cull_Ng", None), getattr(g, "cull_N", None))
        self._packed_keep = keep

    def submit_grids_device(self, ngrids, d_cu, d_cv, d_nkeys, d_flags, d_pbase, d_cbase, d_tbase, d_times,
                            d_P, d_Ci, d_Oi, total_mps, d_culled=None):
        """Device-resident grids: every argument is a device pointer (int)."""
        self._check(self.L.aqh_submit_grids_device(self.ctx, ngrids, d_cu, d_cv, d_nkeys, d_flags, d_pbase,
                                                   d_cbase, d_tbase, d_times, d_P, d_Ci, d_Oi, d_culled, total_mps),
                    "aqh_submit_grids_device")

    def set_mode(self, batched: bool):
        """AQH_MODE_BATCHED (persistent work queue + CUDA graph) or AQH_MODE_PLAIN."""
        self._check(self.L.aqh_set_mode(self.ctx, 1 if batched else 0), "aqh_set_mode")

    def set_tuning(self, tile_pixels: int = 0, supertile_pixels: int = 0, persistent_ctas: int = 0,
                   filter_ctas_per_sm: int = 0):
        """Launch shape of the sampling and filter stages (aqh_set_tuning); zeros are the defaults."""
        t = Tuning(tile_pixels, supertile_pixels, persistent_ctas, filter_ctas_per_sm, 0.0)
        self._check(self.L.aqh_set_tuning(self.ctx, C.byref(t)), "aqh_set_tuning")

    def get_tuning(self) -> dict:
        t = Tuning()
        self._check(self.L.aqh_get_tuning(self.ctx, C.byref(t)), "aqh_get_tuning")
        return {k: getattr(t, k) for k, _ in Tuning._fields_}

    def autotune(self, repeats: int = 3) -> dict:
        """Time the open frame under each candidate launch shape and keep the
        fastest (aqh_autotune); returns the choice with its device ms."""
        t = Tuning()
        self._check(self.L.aqh_autotune(self.ctx, repeats, C.byref(t)), "aqh_autotune")
        return {k: getattr(t, k) for k, _ in Tuning._fields_}

    def set_stream(self, stream_handle: int):
        self._check(self.L.aqh_set_stream(self.ctx, stream_handle or None), "aqh_set_stream")

    def set_cull_normals(self, Ng, N=None):
        """Shade / Split culling for the frame (aqh_set_cull_normals): camera-space
        Ng and N (or None) per P entry."""
        ng = None if Ng is None else np.ascontiguousarray(Ng, np.float32).reshape(-1, 3)
        n = None if N is None else np.ascontiguousarray(N, np.float32).reshape(-1, 3)
        cnt = 0 if ng is None else ng.shape[0]
        self._check(self.L.aqh_set_cull_normals(self.ctx, _p(ng, _f32p), _p(n, _f32p), cnt), "aqh_set_cull_normals")

    def set_host_copy(self, engines: bool):
        """Three-float P by the copy engines (True) or read by a kernel (aqh_set_host_copy)."""
        self._check(self.L.aqh_set_host_copy(self.ctx, 1 if engines else 0), "aqh_set_host_copy")

    def set_imager(self, enabled: bool):
        """aqh_set_imager: frames stop after the filter until apply_imager."""
        self._check(self.L.aqh_set_imager(self.ctx, 1 if enabled else 0), "aqh_set_imager")

    def apply_imager(self, ci_oi):
        """aqh_apply_imager: the imager shader's Ci and Oi, float[pixel][6]."""
        a = np.ascontiguousarray(ci_oi, np.float32).reshape(-1)
        self._check(self.L.aqh_apply_imager(self.ctx, _p(a, _f32p), C.c_size_t(a.size)), "aqh_apply_imager")

    def render(self, sync: bool = True):
        self._check(self.L.aqh_render(self.ctx, 1 if sync else 0), "aqh_render")

    def synchronize(self):
        self._check(self.L.aqh_synchronize(self.ctx), "aqh_synchronize")

    # ---- results ------------------------------------------------------------
    def _dims(self):
        cx0, cx1, cy0, cy1 = self.frame.crop_window
        return cx1 - cx0, cy1 - cy0

    def read_channels(self) -> np.ndarray:
        w, h = self._dims()
        out = np.zeros((h, w, 9), np.float32)
        self._check(self.L.aqh_read_channels(self.ctx, _p(out, _f32p), out.size), "aqh_read_channels")
        return out

    def read_bucket(self, bx: int, by: int) -> np.ndarray:
        bw, bh = C.c_int32(), C.c_int32()
        out = np.zeros(self.frame.bucket[0] * self.frame.bucket[1] * 9, np.float32)
        self._check(self.L.aqh_read_bucket(self.ctx, bx, by, _p(out, _f32p), out.size, C.byref(bw), C.byref(bh)),
                    "aqh_read_bucket")
        return out[:bw.value * bh.value * 9].reshape(bh.value, bw.value, 9)

    def read_quantized(self, channels=(0, 1, 2, 6)) -> np.ndarray:
        w, h = self._dims()
        ch = np.array(channels, np.int32)
        out = np.zeros((h, w, len(ch)), np.uint8)
        self._check(self.L.aqh_read_quantized_u8(self.ctx, _p(ch, _i32p), len(ch), _p(out, _u8p), out.size),
                    "aqh_read_quantized_u8")
        return out

    def dspy_geometry(self) -> DspyGeometry:
        g = DspyGeometry()
        self._check(self.L.aqh_dspy_geometry_of(self.ctx, C.byref(g)), "aqh_dspy_geometry_of")
        return g

    def read_display(self, channels=(0, 1, 2, 6), one=255.0, qmin=0.0, qmax=255.0, dither_amp=0.5, zero=0.0,
                     fmt=0, dither=None) -> np.ndarray:
        """One display request (aqh_read_display): the crop window as
        [h, w, nchan] of the element type the request selects (or `fmt`)."""
        w, h = self._dims()
        d = Display()
        d.nchan = len(channels)
        for i, c in enumerate(channels):
            d.channels[i] = int(c)
        d.q_zero, d.q_one, d.q_min, d.q_max, d.q_dither = zero, one, qmin, qmax, dither_amp
        d.format = int(fmt)
        keep = None
        if dither is not None:
            keep = np.ascontiguousarray(dither, np.float32).reshape(-1)
            d.dither = keep.ctypes.data
        f = fmt or self.L.aqh_display_format(one, qmin, qmax)
        out = np.zeros((h, w, len(channels)), DSPY_DTYPES[f])
        used = C.c_int(0)
        self._check(self.L.aqh_read_display(self.ctx, C.byref(d), out.ctypes.data, out.nbytes, C.byref(used)),
                    "aqh_read_display")
        assert used.value == f
        return out

    def read_samples(self) -> dict:
        x0, y0, w, h = self.frame.sample_region
        n = w * h * self.frame.spp
        r = {"winner": np.zeros(n, np.int32), "occlz": np.zeros(n, np.float32), "nfrag": np.zeros(n, np.int32),
             "valid": np.zeros(n, np.uint8), "sdata": np.zeros((n, 7), np.float32)}
        self._check(self.L.aqh_read_samples(self.ctx, _p(r["winner"], _i32p), _p(r["occlz"], _f32p),
                                            _p(r["nfrag"], _i32p), _p(r["valid"], _u8p), _p(r["sdata"], _f32p), n),
                    "aqh_read_samples")
        return r

    def stats(self) -> dict:
        st = FrameStats()
        self._check(self.L.aqh_get_stats(self.ctx, C.byref(st)), "aqh_get_stats")
        return {k: getattr(st, k) for k, _ in FrameStats._fields_}

    # ---- convenience ----------------------------------------------------------
    def render_scene(self, scene: Scene, qchannels=(0, 1, 2, 6), samples: bool = True) -> dict:
        self.frame_begin(scene.frame)
        self.set_samples(scene.samples)
        self.submit_scene_grids(scene.grids)
        self.render(sync=True)
        res = {"channels": self.read_channels(), "quantized": self.read_quantized(qchannels)}
        if self.naov:
            res["aov"] = self.read_aov()
        if samples:
            res.update(self.read_samples())
        res["stats"] = self.stats()
        return res


# ---------------------------------------------------------------------------
# Serving (aqh_server_*)

class Job(C.Structure):
    _fields_ = [("frame", FrameDesc), ("samples", Samples), ("ngrids", C.c_int),
                ("cu", C.c_void_p), ("cv", C.c_void_p), ("nkeys", C.c_void_p), ("flags", C.c_void_p),
                ("pbase", C.c_void_p), ("cbase", C.c_void_p), ("tbase", C.c_void_p), ("times", C.c_void_p),
                ("ntimes", C.c_size_t), ("P", C.c_void_p), ("nP", C.c_size_t), ("Ci", C.c_void_p),
                ("Oi", C.c_void_p), ("nC", C.c_size_t), ("culled", C.c_void_p), ("micropolygons", C.c_int64),
                ("rgba", C.c_void_p), ("channels", C.c_void_p)]


class JobInfo(C.Structure):
    _fields_ = [("id", C.c_int64), ("status", C.c_int), ("state", C.c_int), ("t_submit", C.c_double),
                ("t_admit", C.c_double), ("t_done", C.c_double), ("footprint", C.c_size_t),
                ("ms_device", C.c_float), ("slot", C.c_int), ("ms_prepare", C.c_float), ("ms_render", C.c_float),
                ("ms_read", C.c_float)]


class ServerOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("hbm_budget", C.c_size_t), ("slots", C.c_int), ("mode", C.c_int),
                ("admission", C.c_int)]


class ServerInfo(C.Structure):
    _fields_ = [("budget", C.c_size_t), ("in_use", C.c_size_t), ("peak_in_use", C.c_size_t),
                ("pending", C.c_int64), ("completed", C.c_int64), ("running", C.c_int), ("peak_running", C.c_int),
                ("graphs_built", C.c_int64), ("rerenders", C.c_int64)]


def _bind_server(L):
    if getattr(L, "_server_bound", False):
        return
    vp = C.c_void_p
    L.aqh_server_create.argtypes = [C.POINTER(ServerOpts), C.POINTER(vp)]
    L.aqh_server_destroy.argtypes = [vp]
    L.aqh_server_destroy.restype = None
    L.aqh_server_submit.argtypes = [vp, C.POINTER(Job), C.POINTER(C.c_int64)]
    L.aqh_server_poll.argtypes = [vp, C.c_int64, C.POINTER(JobInfo)]
    L.aqh_server_wait.argtypes = [vp, C.c_int64, C.c_int, C.POINTER(JobInfo)]
    L.aqh_server_cancel.argtypes = [vp, C.c_int64]
    L.aqh_server_job_error.argtypes = [vp, C.c_int64]
    L.aqh_server_job_error.restype = C.c_char_p
    L.aqh_server_stats.argtypes = [vp, C.POINTER(ServerInfo)]
    L.aqh_job_footprint.argtypes = [C.POINTER(Job)]
    L.aqh_job_footprint.restype = C.c_size_t
    for n in ("aqh_server_create", "aqh_server_submit", "aqh_server_poll", "aqh_server_wait", "aqh_server_cancel",
              "aqh_server_stats"):
        getattr(L, n).restype = C.c_int
    L._server_bound = True


def make_job(scene: Scene, keep: list, want_channels: bool = False):
    """aqh_job for a scene; arrays it points to are appended to `keep`."""
    fr, g, s = scene.frame, scene.grids, scene.samples

    def a(x, dt):
        if x is None:
            return None
        x = np.ascontiguousarray(x, dt)
        keep.append(x)
        return x
    j = Job()
    j.frame = frame_desc(fr)
    j.samples = Samples(int(s.npatterns), _p(a(s.pos, np.float32), _f32p), _p(a(s.time, np.float32), _f32p),
                        _p(a(s.dof, np.float32), _f32p), _p(a(s.shuffle, np.int32), _i32p),
                        _p(a(s.lod, np.float32), _f32p), _p(a(s.pos_index, np.uint32), _u32p),
                        _p(a(s.dof_index, np.uint32), _u32p), _p(a(s.time_index, np.uint32), _u32p),
                        _p(a(s.shuffle_index, np.uint32), _u32p), _p(a(s.lod_index, np.uint32), _u32p),
                        _p(a(s.dither, np.float32), _f32p))
    j.ngrids = g.ngrids
    for k, dt in (("cu", np.int32), ("cv", np.int32), ("nkeys", np.int32), ("flags", np.int32),
                  ("pbase", np.int64), ("cbase", np.int64), ("tbase", np.int32), ("times", np.float32),
                  ("P", np.float32), ("Ci", np.float32), ("Oi", np.float32)):
        setattr(j, k, a(getattr(g, k), dt).ctypes.data)
    j.ntimes = int(g.times.size)
    j.nP = int(g.P.shape[0])
    j.nC = int(g.Ci.shape[0])
    if g.culled is not None:
        j.culled = a(g.culled, np.uint8).ctypes.data
    j.micropolygons = g.micropolygons
    cx0, cx1, cy0, cy1 = fr.crop_window
    rgba = np.zeros((cy1 - cy0, cx1 - cx0, 4), np.uint8)
    keep.append(rgba)
    j.rgba = rgba.ctypes.data
    chans = None
    if want_channels:
        chans = np.zeros((cy1 - cy0, cx1 - cx0, 9), np.float32)
        keep.append(chans)
        j.channels = chans.ctypes.data
    return j, rgba, chans


class Server:
    """aqh_server: jobs admitted by HBM footprint onto `slots` resident contexts."""

    def __init__(self, device: int = 0, budget: int = 0, slots: int = 4, batched: bool = True,
                 admission: str = "arrival"):
        self.L = load()
        _bind_server(self.L)
        self.sv = C.c_void_p()
        adm = {"arrival": 0, "fifo": 0, "smallest": 1}[admission]
        rc = self.L.aqh_server_create(C.byref(ServerOpts(device, budget, slots, 1 if batched else 0, adm)),
                                      C.byref(self.sv))
        if rc != AQH_OK:
            raise AqhError(rc, "aqh_server_create")
        self._jobs = {}

    def close(self):
        if self.sv:
            self.L.aqh_server_destroy(self.sv)
            self.sv = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def footprint(self, scene: Scene) -> int:
        keep = []
        j, _, _ = make_job(scene, keep)
        return int(self.L.aqh_job_footprint(C.byref(j)))

    def submit(self, scene: Scene, want_channels: bool = False) -> int:
        keep = []
        j, rgba, chans = make_job(scene, keep, want_channels)
        jid = C.c_int64()
        rc = self.L.aqh_server_submit(self.sv, C.byref(j), C.byref(jid))
        if rc != AQH_OK:
            raise AqhError(rc, "aqh_server_submit")
        self._jobs[jid.value] = (j, keep, rgba, chans)
        return jid.value

    def wait(self, jid: int, timeout_ms: int = 600000):
        info = JobInfo()
        rc = self.L.aqh_server_wait(self.sv, jid, timeout_ms, C.byref(info))
        return rc, info

    def poll(self, jid: int):
        info = JobInfo()
        rc = self.L.aqh_server_poll(self.sv, jid, C.byref(info))
        return rc, info

    def cancel(self, jid: int) -> int:
        return self.L.aqh_server_cancel(self.sv, jid)

    def error(self, jid: int) -> str:
        return self.L.aqh_server_job_error(self.sv, jid).decode()

    def result(self, jid: int):
        _, _, rgba, chans = self._jobs[jid]
        return rgba, chans

    def release(self, jid: int):
        self._jobs.pop(jid, None)

    def stats(self) -> dict:
        si = ServerInfo()
        self.L.aqh_server_stats(self.sv, C.byref(si))
        return {k: getattr(si, k) for k, _ in ServerInfo._fields_}
