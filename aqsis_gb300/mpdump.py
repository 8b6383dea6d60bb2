"""Micropolygon dump files (CqMPDump, libs/core/mpdump.cpp:40-210) as hider input.

aqsis built with ENABLE_MPDUMP and run with Option "mpdump" "enabled" 1
writes every micropolygon that passes CqImageBuffer::AddMPG's crop test
(imagebuffer.cpp:541-545), with vertex A's colour and opacity, plus each
bucket's pixel sample positions.  `read` parses one through the library
(aqh_mpdump_scan / aqh_mpdump_read); `scene_from_dump` turns it into a Scene
of one-micropolygon grids in the dump's insertion order, constant shading
(the colour is vertex A's, as CqMicroPolygon::colColor gives it) and the
dumped sample positions as explicit per-pixel patterns; `write` writes a
Scene's micropolygons and samples back in the same layout.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
from typing import Optional

import numpy as np

from . import aqh
from . import scene as S


class DumpInfo(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("micropolygons", C.c_int64), ("samples", C.c_int64)]


def _lib():
    L = aqh.load()
    if not getattr(L, "_mpdump_bound", False):
        vp = C.c_void_p
        L.aqh_mpdump_scan.argtypes = [C.c_char_p, C.POINTER(DumpInfo)]
        L.aqh_mpdump_read.argtypes = [C.c_char_p, C.POINTER(DumpInfo), vp, vp, vp, vp, vp]
        L.aqh_mpdump_write.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int64, vp, vp, vp, C.c_int64, vp, vp]
        for n in ("aqh_mpdump_scan", "aqh_mpdump_read", "aqh_mpdump_write"):
            getattr(L, n).restype = C.c_int
        L.aqh_mpdump_last_error.restype = C.c_char_p
        L._mpdump_bound = True
    return L


def _check(L, rc, what):
    if rc != aqh.AQH_OK:
        raise aqh.AqhError(rc, "%s: %s" % (what, L.aqh_mpdump_last_error().decode()))


def read(path: str) -> dict:
    """Every record of a dump: width/height (-1 if absent), P float32[n, 4, 4]
    in grid vertex order, Ci/Oi float32[n, 4], sample_pix int32[m, 3]
    (pixel x, y, sample index) and sample_pos float32[m, 2]."""
    L = _lib()
    info = DumpInfo()
    _check(L, L.aqh_mpdump_scan(path.encode(), C.byref(info)), "aqh_mpdump_scan")
    n, m = info.micropolygons, info.samples
    P = np.zeros((n, 4, 4), np.float32)
    Ci = np.zeros((n, 4), np.float32)
    Oi = np.zeros((n, 4), np.float32)
    pix = np.zeros((m, 3), np.int32)
    pos = np.zeros((m, 2), np.float32)
    _check(L, L.aqh_mpdump_read(path.encode(), C.byref(info), P.ctypes.data, Ci.ctypes.data, Oi.ctypes.data,
                                pix.ctypes.data, pos.ctypes.data), "aqh_mpdump_read")
    return {"width": info.width, "height": info.height, "P": P, "Ci": Ci, "Oi": Oi, "sample_pix": pix,
            "sample_pos": pos}


def grids_from_dump(d: dict) -> S.Grids:
    """One 1x1 grid per dumped micropolygon, in dump order."""
    n = d["P"].shape[0]
    ones = np.ones(n, np.int32)
    opaque = (d["Oi"][:, :3] >= 1.0).all(axis=1)
    flags = np.where(opaque, S.GRID_OPAQUE, 0).astype(np.int32)   # constant shading: vertex A's colour
    Ci = np.repeat(d["Ci"], 4, axis=0)
    Oi = np.repeat(d["Oi"], 4, axis=0)
    return S.Grids(cu=ones.copy(), cv=ones.copy(), nkeys=ones.copy(), flags=flags,
                   pbase=np.arange(n, dtype=np.int64) * 4, cbase=np.arange(n, dtype=np.int64) * 4,
                   tbase=np.zeros(n, np.int32), times=np.zeros(1, np.float32),
                   P=d["P"].reshape(-1, 4).copy(), Ci=Ci, Oi=Oi)


def samples_from_dump(d: dict, frame: S.Frame, fill: Optional[S.Samples] = None) -> tuple:
    """Explicit per-pixel sample positions over the frame's sample region from
    the dump's sample records (offset = position - pixel corner).  Pixels or
    sample indices the dump does not hold take `fill`'s positions (pattern
    index = pixel index), else the centres of a regular xs x ys grid.
    Returns (Samples, mask of the region's samples the dump supplied)."""
    x0, y0, w, h = frame.sample_region
    spp = frame.spp
    if fill is not None and fill.pos_index is None and fill.npatterns == w * h:
        pos = np.array(fill.pos, np.float32).reshape(w * h, spp, 2)
    else:
        xs, ys = frame.xsamples, frame.ysamples
        c = np.array([((i % xs) + 0.5) / xs for i in range(spp)], np.float32)
        r = np.array([((i // xs) + 0.5) / ys for i in range(spp)], np.float32)
        pos = np.broadcast_to(np.stack([c, r], -1), (w * h, spp, 2)).copy()
    have = np.zeros((w * h, spp), bool)
    pix, sp = d["sample_pix"], d["sample_pos"]
    if pix.shape[0]:
        px, py, si = pix[:, 0] - x0, pix[:, 1] - y0, pix[:, 2]
        ok = (px >= 0) & (px < w) & (py >= 0) & (py < h) & (si >= 0) & (si < spp)
        k = py[ok].astype(np.int64) * w + px[ok]
        off = sp[ok] - pix[ok, :2].astype(np.float32)
        pos[k, si[ok]] = off
        have[k, si[ok]] = True
    smp = S.Samples(npatterns=w * h, pos=pos.reshape(w * h * spp, 2))
    if fill is not None:
        smp = dataclasses.replace(fill, npatterns=w * h, pos=smp.pos, pos_index=None)
    return smp, have


def scene_from_dump(path: str, frame: S.Frame, fill: Optional[S.Samples] = None) -> S.Scene:
    """A Scene from a dump file: the frame's options (resolution taken from
    the dump's image record when present), the dumped micropolygons and the
    dumped sample positions."""
    d = read(path)
    if d["width"] > 0:
        frame = dataclasses.replace(frame, width=d["width"], height=d["height"])
    smp, _ = samples_from_dump(d, frame, fill)
    return S.Scene(frame, grids_from_dump(d), smp)


def write(path: str, sc: S.Scene) -> None:
    """Write a Scene's unculled micropolygons (key 0, insertion order; vertex
    A's Ci and Oi) and every sample position of its sample region as a dump."""
    L = _lib()
    g, fr = sc.grids, sc.frame
    quads, col, opa = [], [], []
    mpbase = 0
    for i in range(g.ngrids):
        cu, cv = int(g.cu[i]), int(g.cv[i])
        pb, cb = int(g.pbase[i]), int(g.cbase[i])
        iv, iu = np.meshgrid(np.arange(cv), np.arange(cu), indexing="ij")
        idx = (iv * (cu + 1) + iu).reshape(-1)
        keep = np.ones(idx.size, bool)
        if g.culled is not None:
            keep = g.culled[mpbase:mpbase + cu * cv] == 0
        mpbase += cu * cv
        idx = idx[keep]
        vi = np.stack([idx, idx + 1, idx + cu + 1, idx + cu + 2], -1)
        quads.append(g.P[pb + vi])
        col.append(g.Ci[cb + idx])
        opa.append(g.Oi[cb + idx])
    P = np.ascontiguousarray(np.concatenate(quads) if quads else np.zeros((0, 4, 4)), np.float32)
    Ci = np.ascontiguousarray(np.concatenate(col) if col else np.zeros((0, 4)), np.float32)
    Oi = np.ascontiguousarray(np.concatenate(opa) if opa else np.zeros((0, 4)), np.float32)
    x0, y0, w, h = fr.sample_region
    spp = fr.spp
    s = sc.samples
    pidx = np.arange(w * h) if s.pos_index is None else np.asarray(s.pos_index).reshape(-1)
    off = np.asarray(s.pos, np.float32).reshape(s.npatterns, spp, 2)[pidx]            # [w*h, spp, 2]
    yy, xx = np.divmod(np.arange(w * h), w)
    corner = np.stack([xx + x0, yy + y0], -1).astype(np.float32)
    spos = np.ascontiguousarray((corner[:, None, :] + off).reshape(-1, 2), np.float32)
    spix = np.ascontiguousarray(np.stack([np.repeat(xx + x0, spp), np.repeat(yy + y0, spp),
                                          np.tile(np.arange(spp), w * h)], -1), np.int32)
    _check(L, L.aqh_mpdump_write(path.encode(), fr.width, fr.height, P.shape[0], P.ctypes.data, Ci.ctypes.data,
                                 Oi.ctypes.data, spos.shape[0], spix.ctypes.data, spos.ctypes.data),
           "aqh_mpdump_write")
