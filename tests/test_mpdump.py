"""Micropolygon dump files (CqMPDump layout, libs/core/mpdump.cpp:40-210):
byte layout, round trips through the library's reader and writer, and the
oracle rendering a dumped stream exactly like the scene it came from."""
import dataclasses
import struct

import numpy as np
import pytest

from aqsis_gb300 import scene as S
from tests import scenes_small as SS


@pytest.fixture(scope="module")
def md(aqh_lib):
    from aqsis_gb300 import mpdump
    return mpdump


def constant_shaded(sc):
    g = sc.grids
    g2 = dataclasses.replace(g, flags=(g.flags & ~S.GRID_SMOOTH).astype(np.int32))
    return S.Scene(sc.frame, g2, sc.samples)


def test_hand_written_file_reads(md, tmp_path):
    """A file packed by hand the way CqMPDump::open / dumpImageInfo / dump
    write it: int sizeof(float), then short-tagged records."""
    A, B, C, D = (1.0, 2.0, 3.0), (4.0, 2.5, 3.5), (4.5, 6.0, 4.0), (0.5, 5.5, 4.5)
    col, opa = (0.25, 0.5, 0.75), (1.0, 1.0, 1.0)
    raw = struct.pack("i", 4)
    raw += struct.pack("h", 3) + struct.pack("ii", 32, 24)
    # GetVertices P[0..3] = A, B, C(index+cu+1), D(index+cu+2); written P0 P1 P3 P2
    raw += struct.pack("h", 1) + struct.pack("3f3f3f3f3f3f", *A, *B, *D, *C, *col, *opa)
    raw += struct.pack("h", 2) + struct.pack("iiiff", 7, 5, 3, 7.25, 5.75)
    raw += struct.pack("h", 1) + struct.pack("18f", *range(18))
    p = tmp_path / "hand.mp"
    p.write_bytes(raw)
    d = md.read(str(p))
    assert (d["width"], d["height"]) == (32, 24)
    assert d["P"].shape == (2, 4, 4)
    assert np.array_equal(d["P"][0, :, :3], np.array([A, B, C, D], np.float32))
    assert np.array_equal(d["Ci"][0, :3], np.array(col, np.float32))
    assert np.array_equal(d["Oi"][0, :3], np.array(opa, np.float32))
    assert np.array_equal(d["P"][1, :, :3], np.array([[0, 1, 2], [3, 4, 5], [9, 10, 11], [6, 7, 8]], np.float32))
    assert d["sample_pix"].tolist() == [[7, 5, 3]]
    assert d["sample_pos"].tolist() == [[7.25, 5.75]]


@pytest.mark.parametrize("raw,what", [
    (struct.pack("i", 8), "sizeof"),
    (struct.pack("i", 4) + struct.pack("h", 9), "unknown id"),
    (struct.pack("i", 4) + struct.pack("h", 1) + b"\0" * 10, "truncated"),
])
def test_bad_files_are_rejected(md, tmp_path, raw, what):
    from aqsis_gb300.aqh import AqhError
    p = tmp_path / "bad.mp"
    p.write_bytes(raw)
    with pytest.raises(AqhError, match=what):
        md.read(str(p))


def test_write_layout_and_round_trip(md, tmp_path):
    sc = SS.edge_cases(seed=3)
    p = tmp_path / "scene.mp"
    md.write(str(p), sc)
    raw = p.read_bytes()
    assert struct.unpack_from("i", raw, 0)[0] == 4
    assert struct.unpack_from("=hii", raw, 4) == (3, sc.frame.width, sc.frame.height)
    # first micropolygon record: grid 0, vertices A B D C then vertex A's Ci and Oi
    g = sc.grids
    cu = int(g.cu[0])
    vi = [0, 1, cu + 2, cu + 1]
    want = np.concatenate([g.P[int(g.pbase[0]) + v, :3] for v in vi] + [g.Ci[int(g.cbase[0]), :3],
                                                                        g.Oi[int(g.cbase[0]), :3]])
    off = 4 + 10
    assert struct.unpack_from("h", raw, off)[0] == 1
    got = np.frombuffer(raw, np.float32, 18, off + 2)
    assert np.array_equal(got, want.astype(np.float32))
    d = md.read(str(p))
    nmp = g.micropolygons - (int(g.culled.sum()) if g.culled is not None else 0)
    assert d["P"].shape[0] == nmp
    x0, y0, w, h = sc.frame.sample_region
    assert d["sample_pix"].shape[0] == w * h * sc.frame.spp
    smp, have = md.samples_from_dump(d, sc.frame)
    assert have.all()
    s = sc.samples
    pidx = np.arange(w * h) if s.pos_index is None else np.asarray(s.pos_index)
    want = np.asarray(s.pos, np.float32).reshape(s.npatterns, sc.frame.spp, 2)[pidx]
    yy, xx = np.divmod(np.arange(w * h), w)
    corner = np.stack([xx + x0, yy + y0], -1).astype(np.float32)[:, None, :]
    # the dump holds corner + offset; corner + (that - corner) is that position again
    assert np.array_equal(corner + smp.pos.reshape(w * h, -1, 2), corner + want)


def test_oracle_renders_dump_like_its_scene(md, oracle, tmp_path):
    """A dumped stream replayed as 1x1 grids: same micropolygons in the same
    order, vertex A's colour, the same sample positions -- so the oracle gives
    the constant-shaded original's results bit for bit."""
    sc = constant_shaded(SS.opaque_small(seed=41, scale=0.02))
    sc = S.Scene(sc.frame, dataclasses.replace(sc.grids, culled=None), sc.samples)
    p = tmp_path / "opaque.mp"
    md.write(str(p), sc)
    ds = md.scene_from_dump(str(p), sc.frame)
    assert ds.grids.micropolygons == sc.grids.micropolygons
    a, b = oracle.render(sc), oracle.render(ds)
    for k in ("winner", "occlz", "valid", "channels", "quantized"):
        assert np.array_equal(np.asarray(a[k]).view(np.uint8), np.asarray(b[k]).view(np.uint8)), k


def test_committed_dump_reads_to_its_fixture(md):
    """tests/golden/mpdump_stream.mp (written by make_golden.py) parses to
    exactly the grids and sample positions stored in mpdump_replay.npz."""
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    fx, _ = S.load_scene(os.path.join(here, "mpdump_replay.npz"))
    sc = md.scene_from_dump(os.path.join(here, "mpdump_stream.mp"), fx.frame)
    for k in ("cu", "cv", "nkeys", "flags", "pbase", "cbase", "P", "Ci", "Oi"):
        assert np.array_equal(np.asarray(getattr(sc.grids, k)), np.asarray(getattr(fx.grids, k))), k
    assert np.array_equal(sc.samples.pos, fx.samples.pos)
