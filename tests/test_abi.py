"""The drop-in boundary: libaqh.so builds, loads without a GPU, and exports
every entry point include/aqh.h declares.  Host-only entry points run here."""
import ctypes
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^[A-Za-z_][A-Za-z0-9_ \*]*?\b(aqh_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("aqh_create", "aqh_frame_begin", "aqh_submit_grid", "aqh_render", "aqh_read_bucket"):
        assert must in names


def test_library_exports_every_declared_symbol(aqh_lib):
    lib = ctypes.CDLL(aqh_lib.lib_path())
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_defaults_match_reference_options(aqh_lib):
    d = aqh_lib.FrameDesc()
    aqh_lib.load().aqh_frame_desc_defaults(ctypes.byref(d))
    # libs/core/options.cpp:273-310
    assert (d.width, d.height) == (640, 480)
    assert (d.xsamples, d.ysamples) == (2, 2)
    assert (d.xfilter, d.yfilter) == (2.0, 2.0)
    assert (d.gain, d.gamma) == (1.0, 1.0)
    assert (d.q_one, d.q_min, d.q_max) == (255.0, 0.0, 255.0)
    assert abs(d.q_dither - 0.5) < 1e-7


def test_filter_tables_match_oracle(aqh_lib, oracle):
    # the weight table is host-computed; it must be bit-identical to the oracle's
    for fid in range(8):
        for (xw, yw, xs, ys) in [(2, 2, 4, 4), (3, 3, 8, 8), (1, 1, 6, 6), (4, 4, 2, 3), (2.5, 1.5, 3, 3)]:
            a = aqh_lib.filter_table(fid, xw, yw, xs, ys)
            b = oracle.filter_table(fid, xw, yw, xs, ys)
            assert a.shape == b.shape
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (fid, xw, yw, xs, ys)


def test_display_format_selection(aqh_lib):
    """aqh_display_format follows selectDataFormat (ddmanager.cpp:249-285)."""
    L = aqh_lib.load()
    f = L.aqh_display_format
    assert f(0.0, 0.0, 255.0) == 1                  # no quantize: float32
    assert f(255.0, 0.0, 255.0) == 6                # unsigned 8
    assert f(255.0, 0.0, 256.0) == 4                # unsigned 16
    assert f(65535.0, 0.0, 65535.0) == 4
    assert f(65535.0, 0.0, 65536.0) == 2            # unsigned 32
    assert f(100.0, -128.0, 127.0) == 7             # signed 8
    assert f(100.0, -129.0, 127.0) == 5             # signed 16
    assert f(100.0, -128.0, 128.0) == 5
    assert f(100.0, -32768.0, 32767.0) == 5
    assert f(100.0, -32769.0, 0.0) == 3             # signed 32
