"""ctypes call of aqh_render_noalloc shared by its tests."""
import ctypes as C

import numpy as np


def call_noalloc(lib, scene, d_P, nP, d_Ci, d_Oi, nC, d_out, out_floats, stream, *, pos_index=None, flags=None,
                 pbase=None):
    """Calls aqh_render_noalloc on a scene's grids (host table) with device
    buffers given as integer addresses.  `pos_index`, `flags` and `pbase`
    replace the scene's own arrays when given."""
    from aqsis_gb300 import aqh
    g, s = scene.grids, scene.samples
    desc = aqh.frame_desc(scene.frame)
    err = C.create_string_buffer(512)
    fl = g.flags if flags is None else flags
    pb = g.pbase if pbase is None else pbase
    keep = [np.ascontiguousarray(s.pos, np.float32), np.ascontiguousarray(g.cu, np.int32),
            np.ascontiguousarray(g.cv, np.int32), np.ascontiguousarray(fl, np.int32),
            np.ascontiguousarray(pb, np.int64), np.ascontiguousarray(g.cbase, np.int64)]
    pi = s.pos_index if pos_index is None else pos_index
    pidx = None if pi is None else np.ascontiguousarray(pi, np.uint32)
    f = lib.aqh_render_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(aqh.FrameDesc), C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_size_t,
                  C.c_void_p, C.c_size_t, C.c_void_p, C.c_char_p, C.c_size_t]
    rc = f(C.byref(desc), keep[0].ctypes.data, int(s.npatterns), None if pidx is None else pidx.ctypes.data,
           g.ngrids, keep[1].ctypes.data, keep[2].ctypes.data, keep[3].ctypes.data, keep[4].ctypes.data,
           keep[5].ctypes.data, d_P, nP, d_Ci, d_Oi, nC, d_out, out_floats, stream, err, 512)
    return rc, err.value.decode()
