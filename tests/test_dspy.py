"""Display drivers: the library's Dspy host feeding the capture driver
(bucket and scanline delivery, driver-side format reordering, element
types), on host images; the device path is in test_gpu_display.py."""
import numpy as np
import pytest

from aqsis_gb300 import aqh as A


def read_ppm(path):
    raw = open(path, "rb").read()
    head, rest = raw.split(b"\n", 1)
    assert head == b"P6"
    dims, rest = rest.split(b"\n", 1)
    w, h = (int(v) for v in dims.split())
    mx, rest = rest.split(b"\n", 1)
    assert mx == b"255"
    return np.frombuffer(rest, np.uint8).reshape(h, w, 3)


def read_raw(path):
    raw = open(path, "rb").read()
    head, rest = raw.split(b"\n", 1)
    tag, w, h, n, t = head.split()
    assert tag == b"AQHRAW"
    return int(w), int(h), int(n), int(t), rest


def geometry(w, h, bx=16, by=16):
    return A.DspyGeometry(w, h, 0, 0, w, h, bx, by)


@pytest.fixture(scope="module")
def driver(aqh_lib):
    return A.capture_driver_path()


@pytest.mark.parametrize("scan", [False, True])
def test_buckets_and_scanlines_reach_the_file(driver, tmp_path, scan):
    rng = np.random.default_rng(1)
    w, h = 37, 23
    img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    path = str(tmp_path / "out.ppm")
    dd = A.DisplayDriver(driver, path + ("#scanline" if scan else ""), geometry(w, h, 16, 8), (0, 1, 2, 6),
                         ["r", "g", "b", "a"])
    dd.send_image(img)
    dd.close()
    assert np.array_equal(read_ppm(path), img[..., :3])


def test_driver_reordering_is_followed(driver, tmp_path):
    """The request is a, r, g, b (the reference's rgba display order); the
    capture driver moves r, g, b, a to the front, so the host must permute."""
    rng = np.random.default_rng(2)
    w, h = 20, 18
    img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)   # a, r, g, b
    path = str(tmp_path / "argb.ppm")
    dd = A.DisplayDriver(driver, path, geometry(w, h), (6, 0, 1, 2), ["a", "r", "g", "b"])
    dd.send_image(img)
    dd.close()
    assert np.array_equal(read_ppm(path), img[..., 1:4])


def test_float_display_raw(driver, tmp_path):
    rng = np.random.default_rng(3)
    w, h = 9, 7
    img = rng.random((h, w, 1)).astype(np.float32)
    path = str(tmp_path / "z.raw")
    dd = A.DisplayDriver(driver, path, geometry(w, h, 4, 4), (7,), ["z"], one=0.0, qmin=0.0, qmax=0.0,
                         dither_amp=0.0)
    dd.send_image(img)
    dd.close()
    rw, rh, n, t, data = read_raw(path)
    assert (rw, rh, n, t) == (w, h, 1, 1)
    assert np.array_equal(np.frombuffer(data, np.float32).reshape(h, w, 1), img)


def test_missing_driver_is_an_error(aqh_lib, tmp_path):
    with pytest.raises(A.AqhError):
        A.DisplayDriver(str(tmp_path / "nope.so"), "x.ppm", geometry(4, 4), (0, 1, 2), ["r", "g", "b"])
