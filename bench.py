"""Benchmark of the GB300 hider on the opaque 1080p synthetic stream.

Workload (one "step" = one frame through the whole hider: bin, sample with
early-z and store, combine, filter, exposure, 8-bit quantize):
  1920x1080, 16x16 buckets, PixelSamples 4 4 (stratified-jittered patterns),
  200,000 grids of 16x16 raster-space quads (51.2M micropolygons), vertex
  spacing 1 px +/- 0.3 px, z = U[1,1000] + U[-0.01,0.01]/px slope, Ci ~ U[0,1]^3,
  Oi = 1, gaussian 2x2, exposure 1, quantize 255/0/255 without dither.
The grid inputs (2.8 GB) are far larger than L2 (129 MB), so no flush is
needed between steps.

Legs reported on one JSON line:
  value    micropolygons/s with grids resident in HBM (device-timed, CUDA events)
  e2e      micropolygons/s through the C-ABI from page-locked host arrays
           (P, Ci, Oi as three-float entries, the reference's CqVector3D /
           CqColor layout): per step the H2D copy of every grid array, the
           render and the D2H read of the RGBA8 image are inside the timed region
  roofline achieved GB/s of the sampling kernel (the dominant one) over its
           algorithmic bytes (P, Ci, Oi float4 per vertex, read once) against
           the measured HBM copy bandwidth
  cpu_baseline  the oracle (a restatement of the reference hider) timed
           single-threaded on a bounded slice of the same workload

`--impl reference` times the reference's CPU hider instead: the reference does
not build here (Boost, libtiff, flex and bison are missing), so its oracle
restatement runs, image strips spread over every host core.

Multi-GPU: the hider does not shard a frame across GPUs; `--gpus N` runs N
independent replicas (one per rank) and reports their summed throughput.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "micropolygons/s"
CONFIG = {"workload": "opaque_stream_1080p_16spp", "width": 1920, "height": 1080, "bucket": 16,
          "pixel_samples": [4, 4], "grids": 200000, "grid_quads": [16, 16], "micropolygons": 51_200_000,
          "filter": "gaussian 2x2", "exposure": [1, 1], "quantize": [255, 0, 255, 0],
          "l2": "inputs 2.8 GB >> 129 MB L2 (no flush)"}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def max_over_ranks(x: float, dist, device) -> float:
    """The slowest replica's time: every rank renders its own frame (no
    exchange), so the job takes as long as the slowest one."""
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: float, world: int, ms_max: float) -> float:
    """Whole-job throughput of `world` replicas that each processed
    `units_per_rank` units, timed by the slowest rank."""
    return units_per_rank * world / (ms_max / 1e3)


class ClockSampler:
    """nvidia-smi SM clock and throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    except Exception:
        return {"hbm_gbs": 6800.0, "source": "fallback"}


WORKLOADS = {
    "opaque": ("opaque_stream", 0xC1, {"workload": "opaque_stream_1080p_16spp"}),
    "transparent": ("transparent_stream", 0xC2,
                    {"workload": "transparent_stream_1080p_64spp", "pixel_samples": [8, 8], "grids": 16200,
                     "micropolygons": 4_147_200, "filter": "catmull-rom 3x3",
                     "window": "960x540 centre, ~8 layers", "opacity": "U[0.1,0.9]^3"}),
    "mbdof": ("motion_dof_stream", 0xC3,
              {"workload": "motion_dof_stream_1080p_36spp", "pixel_samples": [6, 6], "grids": 100000,
               "micropolygons": 25_600_000, "filter": "box 1x1", "shutter": [0, 1],
               "dof": {"fstop": 2.8, "focal_length": 0.05, "focal_distance": 50}, "motion_px": 20}),
    "spheres": ("sphere_scene", 0xC0,
                {"workload": "spheres_640x480_16spp", "width": 640, "height": 480, "bucket": 32,
                 "pixel_samples": [4, 4], "filter": "gaussian 2x2", "spheres": 64, "radius": [0.2, 1.0],
                 "z": [5, 30], "shading_rate": 1, "surface": "plastic, one distant light (restated)",
                 "projection": "camera-space grids, projected on the device every frame"}),
}


KERNELS = {"opaque": "sample_opaque_kernel", "transparent": "sample_frag_kernel + resolve_frag_kernel", "mbdof": "sample_mbq_kernel",
           "spheres": "sample_opaque_kernel"}
# kernels one batched frame launches: id table, grid rects, super-tile count,
# scan, super-tile write (binning); the sampler(s); the filter, which also
# quantizes the frame's 8-bit display.  The transparent frame launches the
# occluder scan, both static samplers (one returns at once) and the Combine
# kernel of fragment-only frames (which returns at once when the ordered
# sampler ran); the motion frame the staging-bounds kernel before its sampler.
LAUNCHES = {"opaque": 7, "transparent": 10, "mbdof": 8, "spheres": 8}  # spheres: + the projection
L2_BYTES = 129 << 20
# measured DRAM bytes per micropolygon of the sampler launch (ncu, 0.35 scale)
TRAFFIC_PER_MP = {"opaque": (98.411520e6 + 142.133760e6) / 6_272_000}


def make_scene(args):
    from aqsis_gb300 import scene as S
    fn, seed, _ = WORKLOADS[args.workload]
    if args.workload == "spheres":
        from aqsis_gb300 import spheres
        s = args.scale
        return spheres.sphere_scene(seed=seed, width=max(16, int(640 * s)), height=max(16, int(480 * s)))
    fn = getattr(S, fn)
    if args.scale == 1.0:
        return fn(seed=seed)
    return S.scaled(fn, args.scale, seed=seed)


def cpu_baseline(args) -> dict:
    """Single-threaded oracle on a bounded slice: the same generator scaled so
    the depth complexity stays ~24.7 (about 10 s of CPU work)."""
    from aqsis_gb300 import scene as S
    from oracle import oracle as O
    O.build()
    fn, seed, _ = WORKLOADS[args.workload]
    if args.workload == "spheres":
        from aqsis_gb300 import spheres
        from oracle.oracle import projected_grids
        sc = spheres.sphere_scene(seed=seed)
        sc.grids = projected_grids(sc)  # Split's projection, done before the timed oracle run
    else:
        sc = S.scaled(getattr(S, fn), args.cpu_scale if args.workload == "opaque" else args.cpu_scale / 4,
                      seed=seed)
    t0 = time.perf_counter()
    O.render(sc, want_samples=False)
    dt = time.perf_counter() - t0
    mps = sc.grids.micropolygons
    return {"value": mps / dt, "unit": METRIC, "cores": 1, "kind": "port",
            "sample": "%dx%d, %d grids (%d micropolygons, same density), one frame in %.2f s"
                      % (sc.frame.width, sc.frame.height, sc.grids.ngrids, mps, dt)}


def _close_or_same(a, b, rel=1e-5, abs_=1e-6):
    """Within 1e-5 relative / 1e-6 absolute, or the same non-finite value."""
    with np.errstate(invalid="ignore", over="ignore"):
        d = np.abs(a.astype(np.float64) - b.astype(np.float64))
        ok = (d <= rel * np.abs(b)) | (d <= abs_)
    return ok | (np.isnan(a) & np.isnan(b)) | (np.isinf(a) & (a == b))


def frame_parity(sc, dev_channels, dev_q, qch, e2e_q=None) -> dict:
    """The timed frame against the oracle (a restatement of the reference
    hider) run over the same frame in image strips on every host core, with
    the oracle's float64 twin of compositing and filtering for the error
    figure.  Bars: channels within 1e-5 relative (1e-6 absolute), 8-bit
    values within 1 LSB."""
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    ref = O.render_strips(sc, nthreads=cores, qchannels=qch, want_fp64=True)
    dt = time.perf_counter() - t0
    ok = _close_or_same(dev_channels, ref["channels"])
    q = np.abs(dev_q.astype(np.int64) - ref["quantized"].astype(np.int64))
    bit = bool(np.array_equal(dev_channels.view(np.uint32), ref["channels"].view(np.uint32)))
    with np.errstate(invalid="ignore", divide="ignore"):
        fin = np.isfinite(ref["channels"]) & (np.abs(ref["channels"]) > 1e-6)
        rel = np.abs(dev_channels.astype(np.float64) - ref["channels"]) / np.abs(ref["channels"])
    colour = [0, 1, 2, 3, 4, 5, 6, 8]
    out = {"frame": "the timed frame, %dx%d" % (sc.frame.width, sc.frame.height),
           "oracle": "restatement of the reference hider in %d image strips on %d host threads, %.1f s"
                     % (max(1, min(4 * cores, sc.frame.height)), cores, dt),
           "channels": {"entries": int(ok.size), "outside_bar": int((~ok).sum()), "bit_exact": bit,
                        "max_rel": float(rel[fin].max()) if fin.any() else 0.0},
           "u8_max_lsb": int(q.max()) if q.size else 0,
           "fp64": {"channels": O.fp64_error(dev_channels[..., colour], ref["channels64"][..., colour]),
                    "depth": O.fp64_error(dev_channels[..., 7], ref["channels64"][..., 7])},
           "pass": bool(ok.all() and (q.max() if q.size else 0) <= 1)}
    if e2e_q is not None:
        qe = np.abs(e2e_q.astype(np.int64) - ref["quantized"].astype(np.int64))
        out["e2e_u8_max_lsb"] = int(qe.max()) if qe.size else 0
        out["pass"] = out["pass"] and out["e2e_u8_max_lsb"] <= 1
    return out


def run_reference(args):
    """The reference's CPU hider timed on this machine's host cores: the oracle
    restatement (the reference does not build here) over the same 1080p
    frame, in image strips on one host thread per core (the oracle releases
    the GIL; each strip takes the grids whose bounds reach it, as the
    reference's bucket lists do).  The scene is generated before timing."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    sc = make_scene(argparse.Namespace(workload=args.workload if args.workload != "served" else "opaque",
                                       scale=1.0))
    mps = sc.grids.micropolygons
    times = []
    for step in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        O.render_strips(sc, nthreads=cores, qchannels=(0, 1, 2, 6))
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(dt)
    ms = 1e3 * float(np.mean(times))
    value = mps / (ms / 1e3)
    # the same code on one thread and on every core over a slice of the frame
    from aqsis_gb300 import scene as S
    sl = S.scaled(S.opaque_stream, args.cpu_scale, seed=0xC1)
    t0 = time.perf_counter()
    O.render_strips(sl, nthreads=1, nstrips=1)
    one = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.render_strips(sl, nthreads=cores)
    allc = time.perf_counter() - t0
    cfg = dict(CONFIG, **WORKLOADS.get(args.workload, WORKLOADS["opaque"])[2])
    cfg["grids"], cfg["micropolygons"] = sc.grids.ngrids, mps
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": cfg,
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": "port",
                             "sample": "the whole %dx%d frame (%d micropolygons) per step, %d image strips on %d "
                                       "host threads; scene generated before timing"
                                       % (sc.frame.width, sc.frame.height, mps, max(1, min(4 * cores, sc.frame.height)),
                                          cores)},
            "thread_scaling": {"slice": "%dx%d, %d micropolygons" % (sl.frame.width, sl.frame.height,
                                                                     sl.grids.micropolygons),
                               "one_thread_s": one, "all_threads_s": allc, "threads": cores,
                               "speedup": one / allc},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def resident_leg(sc, local, dev, stream, steps, warmup, autotune, barrier=lambda: None, clocks=None,
                 qch=(0, 1, 2, 6)) -> dict:
    """The device-resident leg: grids uploaded once, then `steps` frames
    timed with CUDA events on the hider's stream (batched form, after the
    autotuner picks the launch shape when `autotune`), plus the plain form
    (one launch per stage).  Returns timings and the last batched frame's
    channels and 8-bit values, read back after the timed region."""
    import torch
    from aqsis_gb300 import aqh, scene as S
    fr, g, smp = sc.frame, sc.grids, sc.samples
    t = {k: torch.from_numpy(np.ascontiguousarray(getattr(g, k))).to(dev)
         for k in ("cu", "cv", "nkeys", "flags", "pbase", "cbase", "tbase", "times", "P", "Ci", "Oi")}
    h = aqh.Hider(local)
    h.set_stream(stream.cuda_stream)
    h.frame_begin(fr)
    h.set_samples(smp)
    h.submit_grids_device(g.ngrids, t["cu"].data_ptr(), t["cv"].data_ptr(), t["nkeys"].data_ptr(),
                          t["flags"].data_ptr(), t["pbase"].data_ptr(), t["cbase"].data_ptr(), t["tbase"].data_ptr(),
                          t["times"].data_ptr(), t["P"].data_ptr(), t["Ci"].data_ptr(), t["Oi"].data_ptr(),
                          g.micropolygons)
    # camera-space grids are projected in place (as Split overwrites P):
    # restore them before every frame, outside the timed region
    cam = bool((np.asarray(g.flags) & S.GRID_CAMERA).any())
    cam_src = (t["P"].clone(), t["flags"].clone()) if cam else None
    # inputs that fit in L2 are evicted between timed frames by writing a buffer twice its size
    flush = torch.empty(2 * L2_BYTES, dtype=torch.uint8, device=dev) if g.nbytes_algorithmic() < 2 * L2_BYTES \
        else None

    def prep():
        with torch.cuda.stream(stream):
            if cam_src is not None:
                t["P"].copy_(cam_src[0])
                t["flags"].copy_(cam_src[1])
            if flush is not None:
                flush.zero_()

    def timed_frames(batched: bool, n: int, w: int):
        h.set_mode(batched)
        for _ in range(w):
            prep()
            h.render(sync=True)
        barrier()
        torch.cuda.synchronize(dev)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
        stage = {"bin": [], "sample": [], "filter": []}
        for i in range(n):
            prep()
            ev[i][0].record(stream)
            h.render(sync=True)
            ev[i][1].record(stream)
            st = h.stats()
            stage["bin"].append(st["ms_bin"])
            stage["sample"].append(st["ms_sample"])
            stage["filter"].append(st["ms_filter"])
        torch.cuda.synchronize(dev)
        barrier()
        lat = [a.elapsed_time(b) for a, b in ev]
        return float(np.mean(lat)), lat, {k: float(np.mean(v)) for k, v in stage.items()}

    plain_ms, plain_lat, plain_stage = timed_frames(False, max(2, steps // 2), 1)
    h.set_mode(True)
    prep()
    tuning = h.autotune(repeats=3) if autotune else dict(h.get_tuning(), ms=None)
    if clocks is not None:
        clocks.start()
    ms, lat, stage = timed_frames(True, steps, warmup)
    clk = clocks.stop() if clocks is not None else None
    res = {"ms": ms, "lat": lat, "stage": stage, "plain_ms": plain_ms, "plain_lat": plain_lat,
           "plain_stage": plain_stage, "tuning": tuning, "clocks": clk,
           "channels": h.read_channels(), "quantized": h.read_quantized(qch), "stats": h.stats()}
    h.close()
    del t
    torch.cuda.empty_cache()
    return res


def sub_workload(name, local, dev, stream, steps, warmup) -> dict:
    """A bounded run of one more configuration in the default bench: its
    full-size frame, device resident, timed like the headline (default launch
    shape), with parity against the oracle: the whole frame for the
    transparent stream and the sphere scene, the 0.1 slice (192x108) for the
    motion blur + depth of field stream, whose full frame the oracle needs
    minutes for."""
    ns = argparse.Namespace(workload=name, scale=1.0)
    t0 = time.perf_counter()
    sc = make_scene(ns)
    gen = time.perf_counter() - t0
    fr, g = sc.frame, sc.grids
    r = resident_leg(sc, local, dev, stream, steps, warmup, autotune=False)
    mps = g.micropolygons
    out = {"config": dict(WORKLOADS[name][2], grids=g.ngrids, micropolygons=mps),
           "ms_per_step": r["ms"], "micropolygons_per_s": mps / (r["ms"] / 1e3),
           "samples_per_s": fr.width * fr.height * fr.spp / (r["ms"] / 1e3),
           "stage_ms": r["stage"], "plain_ms_per_step": r["plain_ms"],
           "frame_latency_ms": {"p50": float(np.percentile(r["lat"], 50)), "p99": float(np.percentile(r["lat"], 99))},
           "kernel": KERNELS[name], "steps": steps, "warmup": warmup, "generation_s": gen,
           "roofline": {"achieved": g.nbytes_algorithmic() / (r["stage"]["sample"] / 1e3) / 1e9, "unit": "GB/s",
                        "frac": g.nbytes_algorithmic() / (r["stage"]["sample"] / 1e3) / 1e9 / peaks()["hbm_gbs"],
                        "algorithmic_bytes": g.nbytes_algorithmic()}}
    if name == "mbdof":
        from aqsis_gb300 import aqh, scene as S
        sl = S.scaled(S.motion_dof_stream, 0.1, seed=0xC3)
        h = aqh.Hider(local)
        h.set_mode(True)
        h.frame_begin(sl.frame)
        h.set_samples(sl.samples)
        h.submit_grids_host(sl.grids)
        h.render(sync=True)
        ch, q = h.read_channels(), h.read_quantized((0, 1, 2, 6))
        h.close()
        out["parity"] = frame_parity(sl, ch, q, (0, 1, 2, 6))
        out["parity"]["frame"] = "the 192x108 slice of the stream (1,000 grids), batched form"
    else:
        out["parity"] = frame_parity(sc, r["channels"], r["quantized"], (0, 1, 2, 6))
    return out


def run_gpu(args):
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()

    from aqsis_gb300 import aqh
    aqh.load(build_if_missing=True)
    sc = make_scene(args)
    fr, g, smp = sc.frame, sc.grids, sc.samples
    mps = g.micropolygons
    G = g.ngrids

    # ---- device-resident leg ----
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(dev)  # the hider's work and the timing events share this stream
    qch = np.array([0, 1, 2, 6], np.int32)
    clocks = ClockSampler(local)
    r = resident_leg(sc, local, dev, stream, args.steps, args.warmup, not args.no_autotune, barrier, clocks,
                     tuple(int(c) for c in qch))
    ms, lat, tuning, clk = r["ms"], r["lat"], r["tuning"], r["clocks"]
    plain_ms, plain_lat = r["plain_ms"], r["plain_lat"]
    ms_max = max_over_ranks(ms, dist, dev)
    value = replica_throughput(mps, world, ms_max)
    launches_per_step = LAUNCHES[args.workload]
    dev_channels, dev_q = r["channels"], r["quantized"]

    # ---- end-to-end leg: host arrays through the C-ABI ----
    import ctypes as C
    # page-locked host arrays; P, Ci and Oi as three-float entries, the layout
    # of the reference's CqVector3D / CqColor grid arrays (aqh_submit_grids_host3)
    pin = {}
    for k in ("cu", "cv", "nkeys", "flags", "pbase", "cbase", "tbase", "times", "P", "Ci", "Oi"):
        a = np.asarray(getattr(g, k))
        if k in ("P", "Ci", "Oi"):
            a = a[:, :3]
        pt = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        pin[k] = pt
    def host_hider(s, engines):
        hh = aqh.Hider(local)
        hh.set_stream(s.cuda_stream)
        hh.set_mode(True)
        hh.set_host_copy(engines)
        hh.set_tuning(tuning["tile_pixels"], tuning["supertile_pixels"], tuning["persistent_ctas"],
                      tuning["filter_ctas_per_sm"])
        hh.frame_begin(fr)
        hh.set_samples(smp)
        L = hh.L
        L.aqh_submit_grids_host3.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 8 + [
            C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_int64]
        L.aqh_submit_grids_host3.restype = C.c_int
        rc = L.aqh_submit_grids_host3(hh.ctx, G, pin["cu"].data_ptr(), pin["cv"].data_ptr(),
                                     pin["nkeys"].data_ptr(), pin["flags"].data_ptr(), pin["pbase"].data_ptr(),
                                     pin["cbase"].data_ptr(), pin["tbase"].data_ptr(), pin["times"].data_ptr(),
                                     int(g.times.size), pin["P"].data_ptr(), int(g.P.shape[0]),
                                     pin["Ci"].data_ptr(), pin["Oi"].data_ptr(), int(g.Ci.shape[0]), None, mps)
        if rc != 0:
            raise RuntimeError("aqh_submit_grids_host3: " + L.aqh_last_error(hh.ctx).decode())
        return hh

    e2e_steps = max(20, args.steps)
    out = np.zeros((fr.height, fr.width, 4), np.uint8)
    # one frame in flight: upload, render and read back per call
    h2 = host_hider(stream, False)
    for _ in range(max(1, args.warmup)):
        h2.render(sync=True)
        out = h2.read_quantized(qch)
    barrier()
    torch.cuda.synchronize(dev)
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(e2e_steps):
        h2.render(sync=False)
        out = h2.read_quantized(qch)
    f1.record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    single_ms = max_over_ranks(f0.elapsed_time(f1) / e2e_steps, dist, dev)
    h2.close()
    # several frames in flight: one context per frame on its own stream, the
    # copy engines bringing later frames' arrays up while one frame samples;
    # every frame still uploads its own inputs and reads back its own image
    k = max(1, args.e2e_inflight)
    streams = [stream] + [torch.cuda.Stream(dev) for _ in range(k - 1)]
    pool = [host_hider(s, True) for s in streams]
    for hh in pool:
        for _ in range(max(1, args.warmup)):
            hh.render(sync=True)
            out = hh.read_quantized(qch)
    n2 = k * e2e_steps
    barrier()
    torch.cuda.synchronize(dev)
    f0.record(stream)
    for i in range(n2):
        hh = pool[i % k]
        if i >= k:
            out = hh.read_quantized(qch)  # frame i-k, before this context renders again
        hh.render(sync=False)
    for i in range(n2 - k, n2):
        out = pool[i % k].read_quantized(qch)
    for s in streams[1:]:
        stream.wait_stream(s)
    f1.record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    multi_ms = max_over_ranks(f0.elapsed_time(f1) / n2, dist, dev)
    for hh in pool:
        hh.close()
    # the faster of the two ways of driving the same API, both measured here
    # (frames in flight lose on hosts whose copy engines share the link badly)
    pipelined = multi_ms <= single_ms
    e2e_ms_max = multi_ms if pipelined else single_ms
    e2e_value = replica_throughput(mps, world, e2e_ms_max)
    h2d = sum(int(p.numel() * p.element_size()) for p in pin.values())
    d2h = int(out.nbytes)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0
    pk = peaks()
    alg_bytes = g.nbytes_algorithmic()  # P + Ci + Oi float4 per vertex, read once
    # DRAM bytes (read + write) of one sampler launch from an ncu capture of the
    # same kernel on a smaller frame of the same stream, scaled by micropolygons
    # (profiles/sample_opaque_kernel_opaque_stream_scale035.md); None where no
    # capture of that kernel exists
    traffic = TRAFFIC_PER_MP[args.workload] * mps if TRAFFIC_PER_MP.get(args.workload) else None
    ms_sample = r["stage"]["sample"]
    achieved = alg_bytes / (ms_sample / 1e3) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / pk["hbm_gbs"], "traffic": traffic,
            "kernel": KERNELS[args.workload], "algorithmic_bytes": alg_bytes,
            "kernel_ms": ms_sample, "peak_source": pk["source"]}
    cfg = dict(CONFIG, **WORKLOADS[args.workload][2], parallelism="replicas" if world > 1 else "single")
    cfg["grids"], cfg["micropolygons"] = G, mps
    if args.workload == "spheres":
        cfg["grid_quads"] = "diced, at most 16x16"
    cfg["l2"] = ("inputs %.1f MB < 2x the 129 MB L2: a %d MB buffer is written between timed frames"
                 % (alg_bytes / 1e6, 2 * L2_BYTES >> 20)) if alg_bytes < 2 * L2_BYTES else \
        "inputs %.2f GB >> 129 MB L2 (no flush)" % (alg_bytes / 1e9)
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": cfg,
            "samples_per_s": fr.width * fr.height * fr.spp * world / (ms_max / 1e3),
            "stage_ms": r["stage"],
            "mode": "batched (persistent tile queue, one CUDA graph per frame)",
            "tuning": tuning,
            "frame_latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
            "plain": {"value": mps * world / (plain_ms / 1e3), "ms_per_step": plain_ms,
                      "frame_latency_ms": {"p50": float(np.percentile(plain_lat, 50)),
                                           "p99": float(np.percentile(plain_lat, 99))}},
            "roofline": roof, "clocks": clk, "gpu_launches": launches_per_step * args.steps,
            "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": e2e_ms_max,
                    "path": "aqh_submit_grids_host3 (P, Ci, Oi as float3) + aqh_render + aqh_read_quantized_u8; " +
                            ("%d contexts, %d frames in flight, copy-engine uploads" % (k, k) if pipelined
                             else "one frame at a time (faster than %d in flight on this host)" % k),
                    "one_in_flight": {"value": replica_throughput(mps, world, single_ms), "ms_per_step": single_ms},
                    "in_flight": {"frames": k, "value": replica_throughput(mps, world, multi_ms),
                                  "ms_per_step": multi_ms}}}
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(args)
    if not args.no_parity:
        line["parity"] = frame_parity(sc, dev_channels, dev_q, tuple(int(c) for c in qch), e2e_q=out)
    if args.workload == "opaque" and not args.no_extra:
        del pin
        torch.cuda.empty_cache()
        line["workloads"] = {}
        for name in ("transparent", "mbdof", "spheres"):
            steps = 5 if name == "mbdof" else 10
            line["workloads"][name] = sub_workload(name, local, dev, stream, steps, 3)
            torch.cuda.empty_cache()
        line["served"] = served_measure(argparse.Namespace(jobs=args.served_jobs, gap_ms=args.gap_ms,
                                                           slots=args.slots, max_mps=args.max_mps,
                                                           slot_mode=args.slot_mode, seed=0xC4,
                                                           admission=args.admission))
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def served_measure(args) -> dict:
    """The served mixed request stream: `args.jobs` distinct requests with
    the configured kinds in proportion (20% motion blur + depth of field, 30%
    transparency, the rest opaque), Poisson arrivals with a mean gap of
    `args.gap_ms`.  Plain = one frame at a time on one context in plain mode
    (one launch per stage); served = the batched server (continuous
    admission onto resident slots, persistent kernels, CUDA graphs).  Both
    submit packed host grids in one call and read back RGBA8.  Reports p50 /
    p99 latency (arrival -> image on the host) under the Poisson schedule and
    frames/s with every request queued at once (saturated), plus the plain
    path's device time per kind."""
    import torch
    from aqsis_gb300 import aqh, scene as S
    aqh.load(build_if_missing=True)
    t0 = time.perf_counter()
    scenes = S.served_stream(args.jobs, seed=args.seed, max_mps=args.max_mps)
    gen_s = time.perf_counter() - t0
    # page-locked copies of every input array (the requests' host buffers)
    for sc in scenes:
        g = sc.grids
        for k in ("P", "Ci", "Oi"):
            setattr(g, k, torch.from_numpy(getattr(g, k)).pin_memory().numpy())
    rng = np.random.default_rng(args.seed + 1)
    gaps = rng.exponential(args.gap_ms / 1e3, args.jobs)
    arrivals = np.cumsum(gaps) - gaps[0]
    mps_total = sum(sc.grids.micropolygons for sc in scenes)

    h = aqh.Hider(0)
    h.set_mode(False)
    sv = aqh.Server(0, slots=args.slots, batched=args.slot_mode == "batched",
                    admission=getattr(args, "admission", "smallest"))
    qch = (0, 1, 2, 6)
    plain_phases = []
    plain_device = []

    def plain_frame(sc):
        """One request the way a served job runs it (packed host grids in one
        call, RGBA8 read back), one frame at a time in plain mode."""
        t0 = time.perf_counter()
        h.frame_begin(sc.frame)
        h.set_samples(sc.samples)
        h.submit_grids_host(sc.grids)
        t1 = time.perf_counter()
        h.render(sync=True)
        t2 = time.perf_counter()
        out = h.read_quantized(qch)
        plain_phases.append((t1 - t0, t2 - t1, time.perf_counter() - t2))
        plain_device.append((sc.kind, h.stats()["ms_total"]))
        return out

    # warm both paths on every request once (context buffers grown, graphs
    # captured), as on a server that has been up for a while
    for sc in scenes:
        plain_frame(sc)
    ids = [sv.submit(sc) for sc in scenes]
    for jid in ids:
        sv.wait(jid)
        sv.release(jid)

    def plain_run(poisson: bool):
        lat = []
        start = time.perf_counter()
        for k, sc in enumerate(scenes):
            arr = arrivals[k] if poisson else 0.0
            now = time.perf_counter() - start
            if poisson and now < arr:
                time.sleep(arr - now)
            plain_frame(sc)
            lat.append(time.perf_counter() - start - arr)
        return time.perf_counter() - start, lat

    def served_run(poisson: bool):
        ids = []
        start = time.perf_counter()
        for k, sc in enumerate(scenes):
            if poisson:
                now = time.perf_counter() - start
                if now < arrivals[k]:
                    time.sleep(arrivals[k] - now)
            ids.append(sv.submit(sc))
        lat, device = [], []
        for jid in ids:
            rc, info = sv.wait(jid)
            if rc != 0:
                raise RuntimeError("served job failed: " + sv.error(jid))
            # the server's own clock: submission (= arrival) to completion
            lat.append(info.t_done - info.t_submit)
            device.append(info.ms_device)
            sv.release(jid)
        return time.perf_counter() - start, lat

    del plain_phases[:], plain_device[:]
    plain_sat, _ = plain_run(False)
    pph = 1e3 * np.mean(np.array(plain_phases), axis=0)
    busy = {}
    for kind, msd in plain_device:
        busy[kind] = busy.get(kind, 0.0) + msd
    served_sat, _ = served_run(False)
    plain_p, plain_lat = plain_run(True)
    served_p, served_lat = served_run(True)
    st = sv.stats()
    sv.close()
    h.close()
    kinds = {k: sum(1 for sc in scenes if sc.kind == k) for k in ("opaque", "transparent", "mb")}
    return {"config": {"workload": "served_mixed_stream", "jobs": args.jobs, "distinct_requests": args.jobs,
                       "mean_gap_ms": args.gap_ms, "slots": args.slots, "slot_mode": args.slot_mode,
                       "admission": getattr(args, "admission", "smallest"), "kinds": kinds,
                       "micropolygons": mps_total, "max_micropolygons": args.max_mps, "generation_s": gen_s},
            "served": {"frames_per_s_saturated": args.jobs / served_sat,
                       "micropolygons_per_s_saturated": mps_total / served_sat,
                       "latency_ms_poisson": {"p50": 1e3 * float(np.percentile(served_lat, 50)),
                                              "p99": 1e3 * float(np.percentile(served_lat, 99))},
                       "peak_jobs_in_flight": st["peak_running"], "peak_hbm_bytes": st["peak_in_use"],
                       "graphs_built": st["graphs_built"], "rerenders": st["rerenders"]},
            "plain": {"frames_per_s_saturated": args.jobs / plain_sat,
                      # share of the saturated run's wall time the device spent on the frames:
                      # near 1 means overlapping requests cannot multiply frames/s
                      "device_busy_fraction": sum(busy.values()) / 1e3 / plain_sat,
                      "micropolygons_per_s_saturated": mps_total / plain_sat,
                      "latency_ms_poisson": {"p50": 1e3 * float(np.percentile(plain_lat, 50)),
                                             "p99": 1e3 * float(np.percentile(plain_lat, 99))},
                      "mean_host_ms": {"prepare": float(pph[0]), "render": float(pph[1]), "read": float(pph[2])},
                      "device_busy_ms_by_kind": busy},
            "speedup_saturated": plain_sat / served_sat}


def run_served(args):
    """`--workload served`: the served stream alone, as its own JSON line."""
    args.seed = 0xC4
    r = served_measure(args)
    line = {"metric": "frames/s", "value": r["served"]["frames_per_s_saturated"], "unit": "frames/s", "n_gpus": 1,
            "steps": args.jobs, "warmup": args.jobs, "ms_per_step": 1e3 / r["served"]["frames_per_s_saturated"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "workload": "served_mixed_stream"}
    line.update(r)
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--scale", type=float, default=1.0, help="scale the workload (1.0 = the full configuration)")
    ap.add_argument("--cpu-scale", type=float, default=0.4)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shape")
    ap.add_argument("--e2e-inflight", type=int, default=3,
                    help="frames in flight in the end-to-end leg (one context each)")
    ap.add_argument("--workload", default="opaque", choices=["opaque", "transparent", "mbdof", "spheres", "served"])
    ap.add_argument("--jobs", type=int, default=256, help="requests of --workload served (all distinct)")
    ap.add_argument("--served-jobs", type=int, default=64, help="requests of the default run's served leg")
    ap.add_argument("--admission", default="smallest", choices=["fifo", "smallest"],
                    help="served admission order among requests that fit")
    ap.add_argument("--no-parity", action="store_true", help="skip the check of the timed frame against the oracle")
    ap.add_argument("--no-extra", action="store_true",
                    help="default run: skip the other workloads and the served leg")
    ap.add_argument("--gap-ms", type=float, default=20.0)
    ap.add_argument("--slots", type=int, default=2)
    ap.add_argument("--max-mps", type=float, default=8e6)
    ap.add_argument("--slot-mode", default="batched", choices=["batched", "plain"],
                    help="served slots: persistent kernel + CUDA graph (batched) or one launch per stage")
    args = ap.parse_args()
    if args.workload == "served":
        sys.exit(run_served(args))
    if args.warmup < 3 and args.impl == "gb300" and args.scale == 1.0:
        args.warmup = 3
    if args.impl == "reference":
        sys.exit(run_reference(args))
    sys.exit(run_gpu(args))


if __name__ == "__main__":
    main()
