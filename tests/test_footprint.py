"""The serving path's HBM footprint estimate (aqh_job_footprint), host only.

The admission of `aqh_server` reserves each job's estimated device memory;
the estimate must cover every buffer a render of the job allocates.  These
tests pin the terms that depend on the kind of job: a transparent job adds
the fragment pool, and a transparent static job (rendered by the
fragment-only sampler) also the per-sample list heads its Combine kernel
reads.  The estimate carries a 10% margin on the total.
"""
import ctypes as C

import numpy as np

from aqsis_gb300 import aqh
from aqsis_gb300 import scene as S
from tests import scenes_small as SS


def _footprint(sc):
    L = aqh.load()
    aqh._bind_server(L)
    keep = []
    j, _, _ = aqh.make_job(sc, keep)
    return int(L.aqh_job_footprint(C.byref(j)))


def _with_flags(sc, opaque):
    g = sc.grids
    flags = np.array(g.flags, dtype=np.int32, copy=True)
    if opaque:
        flags |= S.GRID_OPAQUE
    else:
        flags &= ~np.int32(S.GRID_OPAQUE)
    g.flags = flags
    return sc


def _nsamp(sc):
    _, _, w, h = sc.frame.sample_region
    return w * h * sc.frame.xsamples * sc.frame.ysamples


def _within_margin(diff, terms):
    # the estimate is b + b // 10, so adding `terms` to b adds terms + terms
    # // 10 to it, give or take the one the integer division rounds off
    return terms + terms // 10 <= diff <= terms + terms // 10 + 1


def test_transparent_static_job_adds_pool_and_list_heads(aqh_lib):
    n = _nsamp(SS.opaque_small(seed=21))
    opaque = _footprint(_with_flags(SS.opaque_small(seed=21), True))
    transp = _footprint(_with_flags(SS.opaque_small(seed=21), False))
    pool = max(1 << 20, 2 * n) * 20
    heads = n * 4
    assert _within_margin(transp - opaque, pool + heads)


def test_transparent_motion_job_adds_the_pool_only(aqh_lib):
    # moving jobs keep their fragment lists in the sampler: no list heads
    n = _nsamp(SS.motion_dof_small(seed=22))
    opaque = _footprint(_with_flags(SS.motion_dof_small(seed=22), True))
    transp = _footprint(_with_flags(SS.motion_dof_small(seed=22), False))
    pool = max(1 << 20, 2 * n) * 20
    assert _within_margin(transp - opaque, pool)
