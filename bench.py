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


KERNELS = {"opaque": "sample_opaque_kernel", "transparent": "sample_frag_kernel", "mbdof": "sample_mbp_kernel",
           "spheres": "sample_opaque_kernel"}
# kernels one batched frame launches: id table, grid rects, super-tile count,
# scan, super-tile write (binning); the sampler(s); the filter, which also
# quantizes the frame's 8-bit display.  The transparent frame launches the
# occluder scan and both static samplers, of which one returns at once.
LAUNCHES = {"opaque": 7, "transparent": 9, "mbdof": 7, "spheres": 8}  # spheres: + the projection
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


def _strip_worker(payload):
    """One horizontal strip of the frame through the oracle (crop window)."""
    scale, y0, y1 = payload
    from aqsis_gb300 import scene as S
    from oracle import oracle as O
    sc = S.scaled(S.opaque_stream, scale, seed=0xC1)
    sc.frame.crop = (0, sc.frame.width, y0, y1)
    from aqsis_gb300.scene import make_samples
    sc.samples = make_samples(sc.frame, np.random.default_rng(7), 250)
    t0 = time.perf_counter()
    O.render(sc, want_samples=False)
    return time.perf_counter() - t0


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import multiprocessing as mp
    from aqsis_gb300 import scene as S
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    sc = S.scaled(S.opaque_stream, args.cpu_scale, seed=0xC1)
    h = sc.frame.height
    nstrip = cores
    bounds = [(args.cpu_scale, h * k // nstrip, h * (k + 1) // nstrip) for k in range(nstrip)]
    bounds = [b for b in bounds if b[2] > b[1]]
    ctx = mp.get_context("spawn")
    times = []
    with ctx.Pool(len(bounds)) as pool:
        for step in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            pool.map(_strip_worker, bounds)
            dt = time.perf_counter() - t0
            if step >= args.warmup:
                times.append(dt)
    ms = 1e3 * float(np.mean(times))
    mps = sc.grids.micropolygons
    value = mps / (ms / 1e3)
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": dict(CONFIG, cpu_sample_scale=args.cpu_scale),
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": len(bounds), "kind": "port",
                             "sample": "%dx%d slice of the stream (%d micropolygons, same density) split into "
                                       "%d image strips, one process per host core; includes per-process "
                                       "scene generation" % (sc.frame.width, sc.frame.height, mps, len(bounds))},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


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
    t = {k: torch.from_numpy(np.ascontiguousarray(getattr(g, k))).to(dev)
         for k in ("cu", "cv", "nkeys", "flags", "pbase", "cbase", "tbase", "times", "P", "Ci", "Oi")}
    stream = torch.cuda.Stream(dev)  # the hider's work and the timing events share this stream
    h = aqh.Hider(local)
    h.set_stream(stream.cuda_stream)
    h.frame_begin(fr)
    h.set_samples(smp)
    h.submit_grids_device(G, t["cu"].data_ptr(), t["cv"].data_ptr(), t["nkeys"].data_ptr(), t["flags"].data_ptr(),
                          t["pbase"].data_ptr(), t["cbase"].data_ptr(), t["tbase"].data_ptr(), t["times"].data_ptr(),
                          t["P"].data_ptr(), t["Ci"].data_ptr(), t["Oi"].data_ptr(), mps)
    qch = np.array([0, 1, 2, 6], np.int32)
    from aqsis_gb300 import scene as S
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

    def timed_frames(batched: bool, steps: int, warmup: int):
        """Device time of `steps` frames (CUDA events on the hider's stream
        around each frame; restores and L2 flushes between frames are not
        timed) and per-frame latencies; plain = one launch per stage with host
        round trips."""
        h.set_mode(batched)
        for _ in range(warmup):
            prep()
            h.render(sync=True)
        barrier()
        torch.cuda.synchronize(dev)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        stage = {"bin": [], "sample": [], "filter": []}
        for i in range(steps):
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
        return float(np.mean(lat)), lat, stage

    plain_ms, plain_lat, _ = timed_frames(False, max(2, args.steps // 2), 1)
    # launch shape picked by the autotuner on this frame (batched form), before
    # the timed region; no tuning changes a pixel
    h.set_mode(True)
    prep()
    tuning = h.autotune(repeats=3) if not args.no_autotune else dict(h.get_tuning(), ms=None)
    clocks = ClockSampler(local)
    clocks.start()
    ms, lat, stage = timed_frames(True, args.steps, args.warmup)
    clk = clocks.stop()
    sample_ms, bin_ms, filt_ms = stage["sample"], stage["bin"], stage["filter"]
    ms_max = max_over_ranks(ms, dist, dev)
    value = replica_throughput(mps, world, ms_max)
    launches_per_step = LAUNCHES[args.workload]
    img = h.read_quantized(qch)  # exercise the readback of the resident frame
    h.close()
    del t
    torch.cuda.empty_cache()

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

    e2e_steps = max(1, min(args.steps, 5))
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
    ms_sample = float(np.mean(sample_ms))
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
                 % (alg_bytes / 1e6, 2 * L2_BYTES >> 20)) if flush is not None else \
        "inputs %.2f GB >> 129 MB L2 (no flush)" % (alg_bytes / 1e9)
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": cfg,
            "samples_per_s": fr.width * fr.height * fr.spp * world / (ms_max / 1e3),
            "stage_ms": {"bin": float(np.mean(bin_ms)), "sample": ms_sample, "filter": float(np.mean(filt_ms))},
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
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_served(args):
    """The served mixed request stream: `args.jobs` requests (drawn from
    `args.distinct` generated scenes, cycled), Poisson arrivals with a mean gap
    of `args.gap_ms`.  Plain = one frame at a time on one context in plain mode
    (one launch per stage); served = the batched server (continuous admission
    onto resident slots, persistent kernels, CUDA graphs).  Reports p50/p99
    latency (arrival -> image on the host) under the Poisson schedule and
    frames/s with every request queued at once (saturated)."""
    import torch
    from aqsis_gb300 import aqh, scene as S
    aqh.load(build_if_missing=True)
    rng = np.random.default_rng(0xC4)
    t0 = time.perf_counter()
    scenes = [S.served_job(rng, 1000 + i, max_mps=args.max_mps) for i in range(args.distinct)]
    gen_s = time.perf_counter() - t0
    # page-locked copies of every input array (the requests' host buffers)
    for sc in scenes:
        g = sc.grids
        for k in ("P", "Ci", "Oi"):
            setattr(g, k, torch.from_numpy(getattr(g, k)).pin_memory().numpy())
    order = [i % args.distinct for i in range(args.jobs)]
    gaps = rng.exponential(args.gap_ms / 1e3, args.jobs)
    arrivals = np.cumsum(gaps) - gaps[0]
    mps_total = sum(scenes[i].grids.micropolygons for i in order)

    # warm both paths on every distinct scene (context buffers, graphs, JIT)
    h = aqh.Hider(0)
    h.set_mode(False)
    sv = aqh.Server(0, slots=args.slots, batched=args.slot_mode == "batched")
    qch = (0, 1, 2, 6)

    plain_phases = []

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
        return out

    for sc in scenes:
        plain_frame(sc)
    # every slot meets the requests' sizes before the timed runs (buffers grown,
    # graphs captured), as on a server that has been up for a while
    for _ in range(2):
        ids = [sv.submit(sc) for sc in scenes]
        for jid in ids:
            sv.wait(jid)
            sv.release(jid)

    def plain_run(poisson: bool):
        lat = []
        start = time.perf_counter()
        for k, i in enumerate(order):
            arr = arrivals[k] if poisson else 0.0
            now = time.perf_counter() - start
            if poisson and now < arr:
                time.sleep(arr - now)
            plain_frame(scenes[i])
            lat.append(time.perf_counter() - start - arr)
        return time.perf_counter() - start, lat

    def served_run(poisson: bool):
        ids = []
        start = time.perf_counter()
        for k, i in enumerate(order):
            if poisson:
                now = time.perf_counter() - start
                if now < arrivals[k]:
                    time.sleep(arrivals[k] - now)
            ids.append((sv.submit(scenes[i]), arrivals[k] if poisson else 0.0))
        lat, service, device, phases = [], [], [], []
        for jid, arr in ids:
            rc, info = sv.wait(jid)
            if rc != 0:
                raise RuntimeError("served job failed: " + sv.error(jid))
            # the server's own clock: submission (= arrival) to completion
            lat.append(info.t_done - info.t_submit)
            service.append(info.t_done - info.t_admit)
            device.append(info.ms_device / 1e3)
            phases.append((info.ms_prepare, info.ms_render, info.ms_read))
            sv.release(jid)
        ph = np.mean(np.array(phases), axis=0)
        served_run.breakdown = {"mean_service_ms": 1e3 * float(np.mean(service)),
                                "mean_device_ms": 1e3 * float(np.mean(device)),
                                "mean_prepare_ms": float(ph[0]), "mean_render_ms": float(ph[1]),
                                "mean_read_ms": float(ph[2])}
        return time.perf_counter() - start, lat

    del plain_phases[:]
    plain_sat, _ = plain_run(False)
    pph = 1e3 * np.mean(np.array(plain_phases), axis=0)
    served_sat, _ = served_run(False)
    plain_p, plain_lat = plain_run(True)
    served_p, served_lat = served_run(True)
    st = sv.stats()
    sv.close()
    h.close()
    kinds = {k: sum(1 for i in order if scenes[i].kind == k) for k in ("opaque", "transparent", "mb")}
    line = {"metric": "frames/s", "value": args.jobs / served_sat, "unit": "frames/s", "n_gpus": 1,
            "steps": args.jobs, "warmup": args.distinct, "ms_per_step": 1e3 * served_sat / args.jobs,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "workload": "served_mixed_stream",
            "config": {"workload": "served_mixed_stream", "jobs": args.jobs, "distinct_scenes": args.distinct,
                       "mean_gap_ms": args.gap_ms, "slots": args.slots, "slot_mode": args.slot_mode, "kinds": kinds,
                       "max_micropolygons": args.max_mps, "generation_s": gen_s},
            "served": {"frames_per_s_saturated": args.jobs / served_sat,
                       "micropolygons_per_s_saturated": mps_total / served_sat,
                       "latency_ms_poisson": {"p50": 1e3 * float(np.percentile(served_lat, 50)),
                                              "p99": 1e3 * float(np.percentile(served_lat, 99))},
                       "peak_jobs_in_flight": st["peak_running"], "peak_hbm_bytes": st["peak_in_use"],
                       "graphs_built": st["graphs_built"], "rerenders": st["rerenders"],
                       "poisson_run": served_run.breakdown},
            "plain": {"saturated_run": {"mean_prepare_ms": float(pph[0]), "mean_render_ms": float(pph[1]),
                                        "mean_read_ms": float(pph[2])},
                      "frames_per_s_saturated": args.jobs / plain_sat,
                      "micropolygons_per_s_saturated": mps_total / plain_sat,
                      "latency_ms_poisson": {"p50": 1e3 * float(np.percentile(plain_lat, 50)),
                                             "p99": 1e3 * float(np.percentile(plain_lat, 99))}},
            "speedup_saturated": plain_sat / served_sat}
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
    ap.add_argument("--jobs", type=int, default=256)
    ap.add_argument("--distinct", type=int, default=32)
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
