"""Host-side refusals of aqh_render_noalloc, run without a GPU.

Every check of the no-allocation entry point runs on the host before it
queues anything, so these calls return their status without touching a
device.  The device addresses passed are placeholders: on a machine with a
GPU the tests are skipped, so that a check that stopped firing could never
hand them to a kernel."""
import numpy as np
import pytest

from tests.conftest import HAS_GPU
from tests.noalloc_util import call_noalloc

pytestmark = pytest.mark.skipif(HAS_GPU, reason="placeholder device addresses are only safe without a GPU")

FAKE = 1 << 20  # never dereferenced: each call below is refused first
EINVAL, ELIMIT = 1, 7


@pytest.fixture(scope="module")
def scene():
    from aqsis_gb300 import scene as S
    return S.scaled(S.opaque_stream, 0.05, seed=91)


def _call(lib, sc, **kw):
    g = sc.grids
    nP = kw.pop("nP", g.P.shape[0])
    nC = kw.pop("nC", g.Ci.shape[0])
    out = kw.pop("out_floats", 1 << 24)
    return call_noalloc(lib, sc, FAKE, nP, FAKE, FAKE, nC, FAKE, out, None, **kw)


def test_pattern_choice_beyond_patterns_is_refused(aqh_lib, scene):
    pi = np.array(scene.samples.pos_index, np.uint32)
    pi[len(pi) // 2] = scene.samples.npatterns
    rc, msg = _call(aqh_lib.load(), scene, pos_index=pi)
    assert rc == EINVAL and "pattern choice" in msg, (rc, msg)


@pytest.mark.parametrize("flag", [32, 64, 128, 256])  # camera space, trim outside, cull back faces / transparent
def test_flags_the_form_does_not_carry_out_are_refused(aqh_lib, scene, flag):
    fl = np.array(scene.grids.flags, np.int32)
    fl[3] |= flag
    rc, msg = _call(aqh_lib.load(), scene, flags=fl)
    assert rc == ELIMIT and "not supported" in msg, (rc, msg)


def test_vertices_beyond_P_are_refused(aqh_lib, scene):
    rc, msg = _call(aqh_lib.load(), scene, nP=scene.grids.P.shape[0] - 1)
    assert rc == EINVAL and "out of range" in msg, (rc, msg)
    pb = np.array(scene.grids.pbase, np.int64)
    pb[0] = -1
    rc, msg = _call(aqh_lib.load(), scene, pbase=pb)
    assert rc == EINVAL and "out of range" in msg, (rc, msg)


def test_vertices_beyond_colours_are_refused(aqh_lib, scene):
    rc, msg = _call(aqh_lib.load(), scene, nC=scene.grids.Ci.shape[0] - 1)
    assert rc == EINVAL and "out of range" in msg, (rc, msg)


def test_short_output_is_refused(aqh_lib, scene):
    f = scene.frame
    rc, msg = _call(aqh_lib.load(), scene, out_floats=9 * f.width * f.height - 1)
    assert rc == EINVAL and "output holds" in msg, (rc, msg)
