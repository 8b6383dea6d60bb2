"""Generate the golden fixtures: small seeded scenes with the oracle's outputs.

    python tests/golden/make_golden.py            # rewrite every fixture
    python tests/golden/make_golden.py --check    # compare without writing

Each ``<case>.npz`` holds the scene exactly as the hider consumes it (frame
options, packed grids, sample pattern caches and per-pixel choices; see
``aqsis_gb300.scene.save_scene``) and the oracle's results for it:
per-sample winning micropolygon id, occluding depth, fragment count, valid
flag, the filtered channel buffer and the quantized
display values.  The fixtures are the pinned record of the oracle; the tests
replay them against the oracle (CPU) and against the device hider (GPU).

The reference's own KATs pin the oracle's inverse bilinear, rounding helpers
and random generator (tests/test_oracle_bilinear.py, tests/test_oracle_kats.py);
these fixtures pin everything downstream of them to the oracle's output.
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from aqsis_gb300 import scene as S  # noqa: E402
from tests import scenes_small as SS  # noqa: E402

QCH = (0, 1, 2, 6)
OUT_KEYS = ("winner", "occlz", "nfrag", "valid", "channels", "quantized")


def reference_pattern_scene():
    """A frame sampled with the reference's own multi-jitter caches (250
    patterns of CqMultiJitteredSampler after Reseed(545)) and per-pixel
    pattern choices."""
    from oracle import oracle as O
    fr = S.Frame(width=48, height=32, xsamples=4, ysamples=4, q_dither=0.0)
    rng = np.random.default_rng(31)
    parts = [SS.plane(-2, -2, 26, 18, 40.0, step=2.0, rng=rng, jitter=0.4, zslope=0.02)]
    for _ in range(8):
        parts.append(SS.plane(rng.uniform(0, 40), rng.uniform(0, 26), 5, 5, float(rng.uniform(5, 35)), rng=rng,
                              jitter=0.3))
    pos, _, _ = O.multijitter_tables(4, 4)
    x0, y0, w, h = fr.sample_region
    smp = S.Samples(npatterns=250, pos=pos, pos_index=rng.integers(0, 250, w * h, dtype=np.uint32))
    return S.Scene(fr, S.concat_grids(parts), smp)


def crop_exposure_dither_scene():
    sc = SS.edge_cases(seed=9)
    fr = sc.frame
    fr.crop = (7, 51, 5, 40)
    fr.gain, fr.gamma = 1.7, 2.2
    fr.q_dither = 0.5
    return SS.custom(fr, sc.grids, seed=9, dither=True)


def depth_filter_scene(mode):
    sc = SS.transparent_edge(seed=12)
    sc.frame.depth_filter = mode
    sc.frame.zthreshold = (0.5, 0.5, 0.5)
    sc.frame.display_z = 1
    return sc


def mpdump_scene():
    """A stream replayed from a micropolygon dump file (CqMPDump layout):
    mpdump_stream.mp is written from a small seeded scene of constant-shaded
    opaque and transparent grids, and the fixture is the scene read back
    from it (1x1 grids in dump order, the dumped sample positions)."""
    from aqsis_gb300 import mpdump
    rng = np.random.default_rng(0x3D)
    fr = S.Frame(width=24, height=16, xsamples=2, ysamples=2, filter="gaussian", xfilter=2.0, yfilter=2.0,
                 q_dither=0.0)
    parts = []
    for k in range(8):
        oi = None if k % 2 == 0 else rng.uniform(0.2, 0.9, (49, 3))
        parts.append(SS.plane(rng.uniform(-3, 14), rng.uniform(-3, 8), 6, 6, float(rng.uniform(2, 40)), rng=rng,
                              jitter=0.3, oi=oi, flags=0, step=1.5))
    sc = SS.custom(fr, S.concat_grids(parts), seed=0x3D)
    path = os.path.join(HERE, "mpdump_stream.mp")
    mpdump.write(path, sc)
    return mpdump.scene_from_dump(path, fr)


CASES = {
    "edge_gaussian_4x4": lambda: SS.edge_cases(seed=3),
    "edge_box_3x5": lambda: SS.edge_cases(seed=4, xs=3, ys=5, filt=("box", 1.0, 1.0)),
    "edge_catmullrom_2x2": lambda: SS.edge_cases(seed=5, xs=2, ys=2, filt=("catmull-rom", 3.0, 3.0)),
    "crop_exposure_dither": crop_exposure_dither_scene,
    "opaque_stream_mini": lambda: S.scaled(S.opaque_stream, 0.02, seed=0xC1),
    "transparent_edge_3x3": lambda: SS.transparent_edge(seed=4),
    "transparent_stream_mini": lambda: S.scaled(S.transparent_stream, 0.025, seed=0xC2),
    "depth_filter_midpoint": lambda: depth_filter_scene(1),
    "depth_filter_max": lambda: depth_filter_scene(2),
    "depth_filter_average": lambda: depth_filter_scene(3),
    "motion_dof_mini": lambda: SS.motion_dof_small(seed=0xC3, scale=0.02),
    "motion_only_mini": lambda: SS.motion_dof_small(seed=21, dof=False, xs=4, ys=4, scale=0.02),
    "dof_only_mini": lambda: SS.dof_only_small(seed=22, scale=0.02),
    "motion_transparent_mini": lambda: SS.motion_dof_small(seed=23, xs=3, ys=3, scale=0.02, transparent=True),
    "reference_patterns": reference_pattern_scene,
    "triangular_static": lambda: SS.triangular_small(seed=9),
    "triangular_motion_dof": lambda: SS.triangular(SS.motion_dof_small(seed=10, xs=4, ys=4, scale=0.02), every=2),
    "camera_perspective": lambda: S.to_camera_space(SS.triangular_small(seed=12), every=2),
    "mpdump_replay": mpdump_scene,
    "motion_static_behind_eye": lambda: SS.motion_static_behind_eye(seed=16, transparent=True),
    "output_variables": lambda: S.with_aov(SS.transparent_edge(seed=14), 3, seed=14),
    "output_variables_motion": lambda: S.with_aov(SS.motion_dof_small(seed=15, xs=3, ys=3, scale=0.015,
                                                                      transparent=True), 2, seed=15),
    "camera_motion_ortho": lambda: S.to_camera_space(SS.motion_mixed_small(seed=13, scale=0.012), orthographic=True),
}


def render_case(scene):
    from oracle import oracle as O
    res = O.render(scene, QCH)
    return {k: res[k] for k in OUT_KEYS + ("aov",) if k in res}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--check", action="store_true")
    args = ap.parse_args()
    from oracle import oracle as O
    O.build()
    bad = 0
    for name, fn in CASES.items():
        sc = fn()
        out = render_case(sc)
        path = os.path.join(HERE, name + ".npz")
        if args.check:
            _, old = S.load_scene(path)
            same = all(np.array_equal(np.asarray(out[k]).view(np.uint8), old["o_" + k].view(np.uint8))
                       for k in out)
            print("%-26s %s" % (name, "same" if same else "DIFFERS"))
            bad += not same
        else:
            S.save_scene(path, sc, qchannels=np.array(QCH, np.int32), **{"o_" + k: v for k, v in out.items()})
            print("%-26s %7d samples %6d micropolygons %8d bytes" % (
                name, out["winner"].size, sc.grids.micropolygons, os.path.getsize(path)))
    return 1 if bad else 0


if __name__ == "__main__":
    sys.exit(main())
