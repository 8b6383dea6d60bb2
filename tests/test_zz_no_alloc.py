"""aqh_render_noalloc: the entry point for callers that cannot allocate
device memory (a host whose device memory belongs to another allocator, a
plugin running in someone else's CUDA context).  It must give the same pixels
as the context path, twice in a row (its fixed scratch arrays keep the
previous call's contents), both in a fresh process and after other tests.

The file name sorts last so that a run stopping at the first failure has run
every other test before this one."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL, ABS = 1e-5, 1e-6


def _scene(seed):
    from aqsis_gb300 import scene as S
    # 96x54 display, 4x4 samples, gaussian 2x2: well inside the no-alloc limits
    return S.scaled(S.opaque_stream, 0.05, seed=seed)


def _noalloc(lib, scene, d_P, d_Ci, d_Oi, d_out, stream):
    from aqsis_gb300 import aqh
    g, s = scene.grids, scene.samples
    desc = aqh.frame_desc(scene.frame)
    err = C.create_string_buffer(512)
    keep = [np.ascontiguousarray(a) for a in (s.pos, g.cu, g.cv, g.flags, g.pbase, g.cbase)]
    pidx = None if s.pos_index is None else np.ascontiguousarray(s.pos_index, np.uint32)
    f = lib.aqh_render_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(aqh.FrameDesc), C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_char_p, C.c_size_t]
    rc = f(C.byref(desc), keep[0].ctypes.data, int(s.npatterns), None if pidx is None else pidx.ctypes.data,
           g.ngrids, keep[1].ctypes.data, keep[2].ctypes.data, keep[3].ctypes.data, keep[4].ctypes.data,
           keep[5].ctypes.data, d_P, d_Ci, d_Oi, d_out, stream, err, 512)
    return rc, err.value.decode()


def test_noalloc_matches_context_path_twice(aqh_lib):
    import torch
    sc = _scene(91)
    h = aqh_lib.Hider(0)
    try:
        ref = h.render_scene(sc, samples=False)["channels"]
    finally:
        h.close()
    dev = torch.device("cuda", 0)
    d_P = torch.from_numpy(sc.grids.P).to(dev)
    d_Ci = torch.from_numpy(sc.grids.Ci).to(dev)
    d_Oi = torch.from_numpy(sc.grids.Oi).to(dev)
    out = torch.full(ref.shape, -1.0, dtype=torch.float32, device=dev)
    lib = aqh_lib.load()
    stream = torch.cuda.current_stream(dev).cuda_stream
    for call in range(2):
        out.fill_(-1.0)
        rc, msg = _noalloc(lib, sc, d_P.data_ptr(), d_Ci.data_ptr(), d_Oi.data_ptr(), out.data_ptr(), stream)
        assert rc == 0, msg
        torch.cuda.synchronize(dev)
        got = out.cpu().numpy()
        d = np.abs(got - ref)
        ok = (d <= REL * np.abs(ref)) | (d <= ABS) | ((got == ref) & np.isinf(ref))
        assert ok.all(), "call %d differs at %d entries" % (call, int((~ok).sum()))


def test_noalloc_rejects_oversized_frames(aqh_lib):
    import torch
    from aqsis_gb300 import scene as S
    sc = S.scaled(S.opaque_stream, 0.2, seed=92)  # 384x216 display: beyond the sample-region limit
    dev = torch.device("cuda", 0)
    t = torch.zeros(16, device=dev)
    rc, msg = _noalloc(aqh_lib.load(), sc, t.data_ptr(), t.data_ptr(), t.data_ptr(), t.data_ptr(), 0)
    assert rc == 7 and "exceeds" in msg, (rc, msg)
