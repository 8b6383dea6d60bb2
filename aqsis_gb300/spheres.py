"""The reference-runnable RIB scene as a shaded grid stream: 640x480, 32x32
buckets, PixelSamples 4 4, gaussian 2x2, ShadingRate 1, 64 opaque spheres
(radius U[0.2, 1], centres uniform in the view frustum at z U[5, 30]) with
the "plastic" surface shader (Cs U[0,1]^3) lit by one distant light.

The reference runs this scene through its own RIB parser, quadric dicing and
shading VM; none of that is the hider, and none of it builds here.  This
module restates what the hider receives from it:

* dicing -- CqQuadric::Diceable / EstimateGridSize (geometry/quadrics.cpp:
  259-346): an 8x8 estimate grid (ESTIMATEGRIDSIZE, quadrics.h:37) projected
  to raster space sets the dice rates lceil(8 * longest edge / sqrt(shading
  rate)); a patch with a rate above 16 (the default SqrtGridSize) is split in
  half along the larger rate (CqSphere::PreSubdivide, quadrics.cpp:413-455),
  else diced with CqSphere::DicePoints (quadrics.cpp:457-492) -- points
  radius * (cos theta cos phi, sin theta cos phi, sin phi), theta in degrees
  from ThetaMin to ThetaMax, phi from asin(zmin / r) to asin(zmax / r);
* culling -- patches whose raster bound lies outside the crop window grown
  by half the filter width are dropped, as CqImageBuffer's surface cull does;
* shading -- plastic (shaders/surface/plastic.sl: Ka 1, Kd 0.5, Ks 0.5,
  roughness 0.1) under distantlight (intensity 1, from the eye along +z):
  Ci = Os * (Cs * Kd * diffuse(Nf) + Ks * specular(Nf, V, roughness)), Oi = Os
  = 1, with Nf = faceforward(N, I) and the standard specular lobe
  max(0, Nf.H)^(1 / roughness); ShadingInterpolation constant.

The grids carry camera-space P (AQH_GRID_CAMERA) and the frame holds the
perspective camera-to-raster matrix, so Split's projection runs on the
device.  Shading values are this restatement's, not the reference VM's: the
stream stands in for the scene's shape and size, not for its pixels.
"""
from __future__ import annotations

import math

import numpy as np

from . import scene as S

ESTIMATE = 8        # ESTIMATEGRIDSIZE
GRID_SIDE = 16      # default SqrtGridSize
TOO_LARGE = 10000   # TOOLARGEQUADS


def _dice_points(r, th0, th1, ph0, ph1, nu, nv):
    """CqSphere::DicePoints: float32 points and unit normals [(nv+1)(nu+1), 3]."""
    th = np.linspace(math.radians(th0), math.radians(th1), nu + 1)
    ph = np.linspace(ph0, ph1, nv + 1)
    ct, st = np.cos(th).astype(np.float32), np.sin(th).astype(np.float32)
    cp, sp = np.cos(ph).astype(np.float32), np.sin(ph).astype(np.float32)
    unit = np.stack([ct[None, :] * cp[:, None], st[None, :] * cp[:, None],
                     np.broadcast_to(sp[:, None], (nv + 1, nu + 1))], -1).astype(np.float32)
    return (np.float32(r) * unit).reshape(-1, 3), unit.reshape(-1, 3)


def _to_raster(M, Pc):
    """Row-vector product with the homogeneous divide (x, y and z)."""
    h = Pc @ M[:3, 3] + M[3, 3]
    q = Pc @ M[:3, :3] + M[3, :3]
    return q / h[:, None]


def _estimate(r, c, piece, M, rate):
    """CqQuadric::EstimateGridSize: dice rates from the longest raster edges of
    an 8x8 estimate grid, and the grid's raster bound."""
    th0, th1, ph0, ph1 = piece
    P, _ = _dice_points(r, th0, th1, ph0, ph1, ESTIMATE, ESTIMATE)
    q = _to_raster(M, P.astype(np.float64) + c).reshape(ESTIMATE + 1, ESTIMATE + 1, 3)
    du = ((q[1:, 1:] - q[1:, :-1]) ** 2).sum(-1)     # (u, v) to (u-1, v)
    dv = ((q[:-1, :-1] - q[1:, :-1]) ** 2).sum(-1)   # (u-1, v-1) to (u-1, v)
    s = math.sqrt(rate)
    nu = max(1, int(math.ceil(ESTIMATE * math.sqrt(du.max()) / s)))
    nv = max(1, int(math.ceil(ESTIMATE * math.sqrt(dv.max()) / s)))
    return nu, nv, q[..., 0].min(), q[..., 0].max(), q[..., 1].min(), q[..., 1].max()


def _shade(Pc, N, cs, Ka=1.0, Kd=0.5, Ks=0.5, roughness=0.1):
    """plastic under one distantlight along +z (no ambient light)."""
    I = Pc
    Nn = N / np.linalg.norm(N, axis=1, keepdims=True)
    sgn = np.where((I * Nn).sum(1) < 0, 1.0, -1.0)[:, None]        # faceforward(N, I)
    Nf = Nn * sgn
    V = -I / np.linalg.norm(I, axis=1, keepdims=True)
    L = np.array([0.0, 0.0, -1.0])                                   # towards the light
    diff = np.maximum(0.0, Nf @ L)[:, None]
    H = L[None, :] + V
    H /= np.linalg.norm(H, axis=1, keepdims=True)
    spec = np.maximum(0.0, (Nf * H).sum(1)) ** (1.0 / roughness)
    return cs[None, :] * (Ka * 0.0 + Kd * diff) + Ks * spec[:, None]


def sphere_scene(seed: int = 0xC0, nspheres: int = 64, width: int = 640, height: int = 480,
                 fov: float = 40.0, shading_rate: float = 1.0, explicit_samples: bool = False) -> S.Scene:
    """The 64-sphere RIB scene as camera-space shaded grids (see the module
    docstring), with the build's own stratified sample patterns."""
    rng = np.random.default_rng(seed)
    fr = S.Frame(width=width, height=height, bucket=(32, 32), xsamples=4, ysamples=4, filter="gaussian",
                 xfilter=2.0, yfilter=2.0)
    m = S.camera_to_raster(width, height, fov_deg=fov)
    M = np.asarray(m, np.float64).reshape(4, 4)
    fr = S.dataclasses.replace(fr, camera_to_raster=m)
    f = 1.0 / math.tan(math.radians(fov) / 2)
    aspect = width / height
    xlo, xhi = -0.5 * fr.xfilter, width + 0.5 * fr.xfilter
    ylo, yhi = -0.5 * fr.yfilter, height + 0.5 * fr.yfilter
    cus, cvs, Ps, Cis = [], [], [], []
    for k in range(nspheres):
        r = rng.uniform(0.2, 1.0)
        z = rng.uniform(5.0, 30.0)
        # uniform in the frustum at depth z: screen x in [-aspect, aspect], y in [-1, 1]
        c = np.array([rng.uniform(-aspect, aspect) * z / f, rng.uniform(-1, 1) * z / f, z])
        cs = rng.uniform(0, 1, 3)
        stack = [(0.0, 360.0, -math.pi / 2, math.pi / 2)]
        while stack:
            piece = stack.pop()
            nu, nv, x0, x1, y0, y1 = _estimate(r, c, piece, M, shading_rate)
            if x1 < xlo or x0 > xhi or y1 < ylo or y0 > yhi:
                continue
            if nu > GRID_SIDE or nv > GRID_SIDE or nu * nv > TOO_LARGE:
                th0, th1, ph0, ph1 = piece
                if nu > nv:
                    tm = (th0 + th1) * 0.5
                    stack += [(tm, th1, ph0, ph1), (th0, tm, ph0, ph1)]
                else:
                    pm = (ph0 + ph1) * 0.5
                    stack += [(th0, th1, pm, ph1), (th0, th1, ph0, pm)]
                continue
            P, N = _dice_points(r, *piece, nu, nv)
            Pc = P.astype(np.float64) + c
            Ci = _shade(Pc, N.astype(np.float64), cs)
            P4 = np.zeros((P.shape[0], 4), np.float32)
            P4[:, :3] = Pc.astype(np.float32)
            C4 = np.zeros((P.shape[0], 4), np.float32)
            C4[:, :3] = Ci.astype(np.float32)
            cus.append(nu)
            cvs.append(nv)
            Ps.append(P4)
            Cis.append(C4)
    G = len(cus)
    Oi = [np.concatenate([np.ones((p.shape[0], 3), np.float32), np.zeros((p.shape[0], 1), np.float32)], 1)
          for p in Ps]
    flags = np.full(G, S.GRID_OPAQUE | S.GRID_CAMERA, np.int32)   # constant shading
    g = S._pack(np.array(cus), np.array(cvs), np.ones(G, np.int32), flags, np.concatenate(Ps),
                np.concatenate(Cis), np.concatenate(Oi))
    smp = S.make_samples(fr, rng, 64, explicit_samples, False)
    sc = S.Scene(fr, g, smp)
    sc.kind = "spheres"
    return sc
