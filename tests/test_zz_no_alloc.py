"""aqh_render_noalloc: the entry point for callers that cannot allocate
device memory (a host whose device memory belongs to another allocator, a
plugin running in someone else's CUDA context).  It must give the same pixels
as the context path, twice in a row (its fixed scratch arrays keep the
previous call's contents), both in a fresh process and after other tests.

The file name sorts last so that a run stopping at the first failure has run
every other test before this one."""
import numpy as np
import pytest

from tests.noalloc_util import call_noalloc

pytestmark = pytest.mark.gpu

REL, ABS = 1e-5, 1e-6


def _scene(seed):
    from aqsis_gb300 import scene as S
    # 96x54 display, 4x4 samples, gaussian 2x2: well inside the no-alloc limits
    return S.scaled(S.opaque_stream, 0.05, seed=seed)


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
        rc, msg = call_noalloc(lib, sc, d_P.data_ptr(), d_P.shape[0], d_Ci.data_ptr(), d_Oi.data_ptr(),
                               d_Ci.shape[0], out.data_ptr(), out.numel(), stream)
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
    # a full-size output, so that only the sample-region limit can refuse the call
    out = torch.zeros(sc.frame.width * sc.frame.height * 9, device=dev)
    rc, msg = call_noalloc(aqh_lib.load(), sc, t.data_ptr(), 4, t.data_ptr(), t.data_ptr(), 4, out.data_ptr(),
                           out.numel(), 0)
    assert rc == 7 and "exceeds" in msg, (rc, msg)


def test_noalloc_refusal_then_render(aqh_lib):
    """A refused call (a flag the form does not carry out) queues nothing, and
    the next good call still gives the context path's pixels.  The buffers
    are real and full-size, so even a missed refusal could not read out of
    bounds."""
    import torch
    sc = _scene(93)
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
    fl = np.array(sc.grids.flags, np.int32)
    fl[0] |= 32  # AQH_GRID_CAMERA
    args = (d_P.data_ptr(), d_P.shape[0], d_Ci.data_ptr(), d_Oi.data_ptr(), d_Ci.shape[0], out.data_ptr(),
            out.numel(), stream)
    rc, msg = call_noalloc(lib, sc, *args, flags=fl)
    assert rc == 7 and "not supported" in msg, (rc, msg)
    torch.cuda.synchronize(dev)
    assert bool((out == -1.0).all()), "a refused call wrote the output"
    rc, msg = call_noalloc(lib, sc, *args)
    assert rc == 0, msg
    torch.cuda.synchronize(dev)
    got = out.cpu().numpy()
    d = np.abs(got - ref)
    ok = (d <= REL * np.abs(ref)) | (d <= ABS) | ((got == ref) & np.isinf(ref))
    assert ok.all(), "differs at %d entries" % int((~ok).sum())
