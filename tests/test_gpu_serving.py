"""Serving: jobs of different resolutions, sample counts and blur settings
in flight together.  Each result must equal the same job rendered alone
(bit-exact here; the stated tolerance is 1e-5 relative / 1 LSB), admission
must respect the HBM budget, and oversize, cancelled and timed-out requests
report the documented statuses."""
import numpy as np
import pytest

from tests import scenes_small as SS

pytestmark = pytest.mark.gpu

AQH_OK, AQH_ETIMEDOUT, AQH_EREJECTED, AQH_ENOTREADY = 0, 4, 5, 6


def mixed_scenes():
    from aqsis_gb300 import scene as S
    return [SS.opaque_small(seed=201), SS.transparent_small(seed=202), SS.motion_dof_small(seed=203),
            SS.edge_cases(seed=204, xs=3, ys=3), S.scaled(S.opaque_stream, 0.08, seed=205),
            SS.dof_only_small(seed=206), SS.transparent_edge(seed=207), SS.opaque_small(seed=208, explicit=True)]


def alone(aqh_lib, sc):
    h = aqh_lib.Hider(0)
    try:
        res = h.render_scene(sc, samples=False)
        return h.read_quantized((0, 1, 2, 6)), res["channels"]
    finally:
        h.close()


@pytest.mark.parametrize("batched,admission", [(True, "arrival"), (False, "arrival"), (True, "smallest")],
                         ids=["batched", "plain-slots", "batched-smallest-first"])
def test_results_same_alone_and_in_the_mix(aqh_lib, batched, admission):
    scenes = mixed_scenes()
    refs = [alone(aqh_lib, sc) for sc in scenes]
    sv = aqh_lib.Server(0, slots=4, batched=batched, admission=admission)
    try:
        ids = [sv.submit(sc, want_channels=True) for sc in scenes]
        for jid, (ref8, refc) in zip(ids, refs):
            rc, info = sv.wait(jid)
            assert rc == AQH_OK, sv.error(jid)
            rgba, chans = sv.result(jid)
            assert np.array_equal(rgba, ref8)
            same = (chans.view(np.uint32) == refc.view(np.uint32)) | (np.isnan(chans) & np.isnan(refc))
            assert same.all()
        st = sv.stats()
        assert st["completed"] == len(scenes)
        assert st["peak_running"] >= 2  # jobs did overlap
    finally:
        sv.close()


def test_admission_respects_budget(aqh_lib):
    scenes = mixed_scenes()
    probe = aqh_lib.Server(0, slots=1)
    fps = [probe.footprint(sc) for sc in scenes]
    probe.close()
    budget = max(fps) + min(fps)  # never more than a couple of jobs at once
    sv = aqh_lib.Server(0, budget=budget, slots=6)
    try:
        ids = [sv.submit(sc) for sc in scenes]
        for jid in ids:
            rc, _ = sv.wait(jid)
            assert rc == AQH_OK, sv.error(jid)
        st = sv.stats()
        assert st["peak_in_use"] <= budget
        assert st["in_use"] == 0
    finally:
        sv.close()


def test_oversize_job_is_rejected(aqh_lib):
    sc = SS.opaque_small(seed=211)
    sv = aqh_lib.Server(0, budget=1 << 20, slots=1)
    try:
        with pytest.raises(aqh_lib.AqhError) as e:
            sv.submit(sc)
        assert e.value.status == AQH_EREJECTED
    finally:
        sv.close()


def test_cancel_and_timeout(aqh_lib):
    from aqsis_gb300 import scene as S
    big = S.scaled(S.opaque_stream, 0.5, seed=221)
    small = SS.opaque_small(seed=222)
    sv = aqh_lib.Server(0, slots=1)
    try:
        a = sv.submit(big)
        b = sv.submit(small)
        c = sv.submit(small)
        rc, info = sv.wait(c, timeout_ms=0)
        assert rc in (AQH_ETIMEDOUT, AQH_OK)
        cancelled = sv.cancel(c)
        if cancelled == AQH_OK:
            rc, info = sv.wait(c, timeout_ms=1000)
            assert info.state == 4 and rc == AQH_EREJECTED
        for jid in (a, b):
            rc, _ = sv.wait(jid)
            assert rc == AQH_OK, sv.error(jid)
    finally:
        sv.close()


def test_smallest_first_admits_small_jobs_ahead(aqh_lib):
    """With one slot and AQH_ADMIT_SMALLEST, small jobs queued behind a large
    pending one are admitted before it (within the aging limit)."""
    from aqsis_gb300 import scene as S
    busy = S.scaled(S.opaque_stream, 0.5, seed=231)
    large = S.scaled(S.opaque_stream, 0.4, seed=232)
    smalls = [SS.opaque_small(seed=233 + i) for i in range(3)]
    sv = aqh_lib.Server(0, slots=1, admission="smallest")
    try:
        first = sv.submit(busy)           # occupies the slot
        big = sv.submit(large)
        little = [sv.submit(sc) for sc in smalls]
        infos = {}
        for jid in [first, big] + little:
            rc, info = sv.wait(jid)
            assert rc == AQH_OK, sv.error(jid)
            infos[jid] = info
        # every small job was admitted no later than the large one, unless the
        # large one aged past the limit while the first job ran
        waited = (infos[big].t_admit - infos[big].t_submit) * 1e3
        if waited < 250:  # AQH_ADMIT_MAX_WAIT_MS
            assert all(infos[j].t_admit <= infos[big].t_admit for j in little)
    finally:
        sv.close()


def test_bad_admission_order_is_refused(aqh_lib):
    import ctypes as C
    L = aqh_lib.load()
    aqh_lib._bind_server(L)
    sv = C.c_void_p()
    rc = L.aqh_server_create(C.byref(aqh_lib.ServerOpts(0, 0, 1, 1, 7)), C.byref(sv))
    assert rc == 1 and not sv.value
