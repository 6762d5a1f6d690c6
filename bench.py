"""Benchmark: frames/s of the per-fragment path on a seeded synthetic scene.

Default workload: config 2 -- 1920x1080 Blinn-Phong pass with trilinear
albedo, tangent-space normal map and 3x3 PCF, preceded by a 2048^2 FP32
shadow pass, 64 seeded meshes (~200k triangles).  One step renders a fixed
batch of K frames (both passes each; K per workload in FRAMES_PER_STEP, 50 at
config 2, stated in config.frames_per_step), every frame timed alone after an
L2 scrub; the workload's schedule is the one pinned for it
(puresoft3d_gb300.autotune.PINNED) unless --autotune or --bin-width is given.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--config c1|c2|c3]
                  [--impl ours|reference]

Arms
  ours       value: frames/s with everything resident in HBM, frame = one
             replay of the recorded command buffer (a CUDA graph running every
             kernel of both passes: vertex set-up, binning, raster, shade);
             CUDA events on the pipeline's stream around each frame, the L2
             scrubbed (256 MB written) before each timed frame.
             e2e: the same through the public API with host buffers: each step
             copies the frame's draw descriptors and uniforms from pinned host
             memory and copies the BGRA8 frame back to pinned host memory;
             steps are issued back to back, alternating between two
             pipelines (double buffering), the L2 scrubbed before each step
             inside the timed region, and the host waits after the last
             ("one_at_a_time": one pipeline, waiting for each frame's
             read-back before the next step).
  reference  the reference pipeline's CPU path (the oracle port of it, on all
             host cores), a bounded sample of frames of the same workload.

With --gpus N (launched by torch.distributed.run) each rank renders its own
replica of the scene on its own GPU ("replicas only": a frame is ordered per
pixel and does not shard); value = all ranks' frames / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

RANK = int(os.environ.get("RANK", "0"))
WORLD = int(os.environ.get("WORLD_SIZE", "1"))
LOCAL_RANK = int(os.environ.get("LOCAL_RANK", "0"))
if WORLD > 1:  # one GPU per rank: make it device 0 of this process before CUDA starts
    os.environ["CUDA_VISIBLE_DEVICES"] = str(LOCAL_RANK)

import numpy as np  # noqa: E402

CONFIGS = {
    "c1": dict(desc="c1: 640x480, one 32x16 UV sphere (992 triangles), 256^2 texture, LIT1 bilinear REPEAT",
               args={}),
    "c2": dict(desc="c2: 1920x1080 LIT2 pass (trilinear albedo, FP16 normal map, 3x3 PCF) after a 2048^2 FP32 "
                    "shadow pass; 64 seeded meshes, ~200k triangles; 4x1024^2 albedo + 1024^2 normal mip chains",
               args={}),
    "c3": dict(desc="c3: 3840x2160 LIT3, 256 seeded meshes, ~2M triangles in 4 depth layers, 16x2048^2 trilinear",
               args={}),
    "c3s": dict(desc="c3s (profiling case): 1920x1080 LIT3, 128 meshes, ~500k triangles, 4x2048^2 trilinear",
                args={}),
    "c5": dict(desc="c5: serving -- 2000 seeded jobs, Poisson arrivals, resolution uniform over 256^2, 512^2, "
                    "1024^2, 1920x1080; meshes from a resident pool of 128 (1k-500k triangles log-uniform), 64 "
                    "resident 512^2 mip chains, LIT3; continuous batching into two 4096^2 atlas slots",
               args={}),
    "c4": dict(desc="c4: 4096 independent 128x128 views (own seeded mesh, 100-5000 triangles log-uniform, own "
                    "orbit camera, own 256^2 texture, LIT1), batched into tiles of an 8192^2 atlas in one pass",
               args={}),
}


# DRAM bytes (read + write) of one launch of a kernel class on each workload
# at its pinned schedule, from one ncu capture of the same kernels on the
# same full-size workload (one-pass metrics dram__bytes_read.sum and
# dram__bytes_write.sum, every launch of two immediate-path frames:
# bench.py --config cN --ncu-frames 2); averages over the launches that ran
# to completion.  c4's are the immediate path's (one launch per frame over
# the whole atlas), the same kernels as the batched pass.
KERNEL_TRAFFIC = {"c1": {"raster": 70272, "shade": 747264}, "c2": {"raster": 5207872, "shade": 18389504},
                  "c3": {"raster": 117094912, "shade": 338297984},
                  "c4": {"raster": 825424640, "shade": 2104926976}}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            m = json.load(f)
        return float(m["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """SM clocks and throttle reasons sampled during the timed region: NVML
    through ctypes every millisecond (reads only), else nvidia-smi."""

    # NVML clocks-event reason bits
    REASONS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown", 0x4: "sw_power_cap"}

    def __init__(self):
        self.samples = []      # (sm_mhz, reasons bitmask)
        self.max_mhz = None
        self.stop_flag = threading.Event()
        self.thread = None
        self.nvml = None
        self.proc = None
        self.lines = []

    def _nvml_open(self):
        import ctypes
        for name in ("libnvidia-ml.so.1", "libnvidia-ml.so"):
            try:
                lib = ctypes.CDLL(name)
                break
            except OSError:
                lib = None
        if lib is None or lib.nvmlInit_v2() != 0:
            return False
        idx = int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or 0)
        h = ctypes.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(idx, ctypes.byref(h)) != 0:
            return False
        mx = ctypes.c_uint()
        if lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0:  # NVML_CLOCK_SM
            self.max_mhz = float(mx.value)
        reasons = None
        for fn in ("nvmlDeviceGetCurrentClocksEventReasons", "nvmlDeviceGetCurrentClocksThrottleReasons"):
            try:
                reasons = getattr(lib, fn)
                break
            except AttributeError:
                continue
        self.nvml = (lib, h, reasons)
        return True

    def _nvml_loop(self):
        import ctypes
        lib, h, reasons = self.nvml
        clk, rs = ctypes.c_uint(), ctypes.c_ulonglong()
        while not self.stop_flag.is_set():
            r = lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk))
            rs.value = 0
            if reasons is not None:
                reasons(h, ctypes.byref(rs))
            if r == 0:
                self.samples.append((float(clk.value), int(rs.value)))
            time.sleep(0.001)

    def start(self):
        try:
            if self._nvml_open():
                self.thread = threading.Thread(target=self._nvml_loop, daemon=True)
                self.thread.start()
                return
        except Exception:
            self.nvml = None
        try:
            q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                          "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                          "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._smi_loop, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _smi_loop(self):
        bits = [0x8, 0x40, 0x20, 0x4]
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 6:
                continue
            try:
                mhz, self.max_mhz = float(parts[0]), float(parts[1])
            except ValueError:
                continue
            m = 0
            for b, v in zip(bits, parts[2:6]):
                if v.lower() == "active":
                    m |= b
            self.samples.append((mhz, m))

    def stop(self):
        self.stop_flag.set()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": [], "samples": 0,
                    "source": "nvml" if self.nvml else ("nvidia-smi" if self.proc else "unavailable")}
        reasons = set()
        for _, m in self.samples:
            for b, n in self.REASONS.items():
                if m & b:
                    reasons.add(n)
        return {"sm_mhz": statistics.median(x for x, _ in self.samples), "sm_max_mhz": self.max_mhz,
                "reasons": sorted(reasons), "samples": len(self.samples), "source": "nvml" if self.nvml else "nvidia-smi"}


# Frames per timed step, per workload: enough that the timed region (and the
# clock samples taken during it) lasts a few hundred milliseconds.
FRAMES_PER_STEP = {"c1": 200, "c2": 50, "c3": 10, "c3s": 20, "c4": 4}


def frames_per_step(args):
    return args.frames_per_step or FRAMES_PER_STEP.get(args.config, 1)


def make_scene(cfg, views=4096):
    from puresoft3d_gb300 import scenes as S
    if cfg == "c4":
        return S.scene_c4(views=views)[0]
    if cfg == "c3s":
        return S.scene_c3(width=1920, height=1080, meshes=128, tri_target=500_000, textures=4)
    return {"c1": S.scene_c1, "c2": S.scene_c2, "c3": S.scene_c3}[cfg]()


SCHED_KEYS = ("bin_width", "raster_occupancy", "span_culling", "row_split", "warp_bins", "span_items",
              "lazy_varyings")


def _sched_dict(s, source):
    from puresoft3d_gb300.autotune import _sched
    d = dict(zip(SCHED_KEYS, _sched(s)))
    d["source"] = source
    return d


def _flag_schedule(args):
    return (args.bin_width, args.raster_occupancy, args.span_culling, args.row_split, args.warp_bins,
            args.span_items, args.lazy_varyings)


def autotune(pipe, record, key, args, pinned=None):
    """The schedule the workload is timed at, applied to `pipe`: the flags'
    (--bin-width ...) when given; else, with --autotune, the fastest
    candidate timed on the frame itself (puresoft3d_gb300.autotune;
    untimed); else the schedule pinned for the workload
    (puresoft3d_gb300.autotune.PINNED), so that its profiles under profiles/
    describe the same kernels."""
    from puresoft3d_gb300.autotune import Autotuner, apply
    if args.bin_width:
        s = _flag_schedule(args)
        apply(pipe, s)
        return _sched_dict(s, "flags")
    if pinned is not None and not args.autotune:
        apply(pipe, pinned)
        return _sched_dict(pinned, "pinned")
    best, ms = Autotuner().tune(pipe, record, key, reps=3)
    d = _sched_dict(best, "autotuner")
    d["candidate_ms"] = {k: round(v, 4) for k, v in ms.items()}
    return d


def twin(scene, tune):
    """A second pipeline with `scene`'s resources and the same schedule."""
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.autotune import apply
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    p = PuresoftPipeline(scene.width, scene.height)
    S.replay_setup(scene, p)
    apply(p, tuple(tune[k] for k in SCHED_KEYS))
    p.finish()
    return p


def e2e_pipelined(pipes, record, hosts, steps):
    """Seconds for `steps` end-to-end steps through the public API, issued
    back to back and alternating between the given pipelines (double
    buffering: one frame's read-back overlaps the next frame's rendering).
    Each pipeline records the frame once as a command buffer together with a
    read-out of its whole colour buffer into its own pinned host array; each
    submission uploads the frame's inputs (draw descriptors, uniforms) from
    pinned host memory, renders and copies the result to the host; the L2 is
    scrubbed (256 MB written) before each step, inside the timed region.
    The host waits once, after the last step."""
    cbs = []
    for pipe, host in zip(pipes, hosts):
        h, w = host.shape[:2]
        pipe.beginCommands()
        record(pipe)
        pipe.copyColourRect(0, 0, w, h, host.ctypes.data, w * 4)
        cbs.append(pipe.endCommands())
    try:
        for _ in range(2):
            for cb, pipe in zip(cbs, pipes):
                cb.submit(upload_inputs=True)
                pipe.finish()
        t0 = time.perf_counter()
        for i in range(steps):
            pipes[i % len(pipes)].scrubL2()  # as between timed device frames; its time counts here
            cbs[i % len(cbs)].submit(upload_inputs=True)
        for pipe in pipes:
            pipe.finish()
        return time.perf_counter() - t0
    finally:
        for cb in cbs:
            cb.destroy()


def run_c4(args):
    """Config 4: images/s of the batched pass (every view in one pass over
    an atlas, replayed as one CUDA graph) against the plain path (one pass
    per view in a 128x128 pipeline, the frame copied out after each view),
    both with every mesh and texture resident."""
    import torch
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline, KERNELS
    views = args.views
    batched, plain = S.scene_c4(views=views)
    size = batched.info["view_size"]
    pipe = PuresoftPipeline(batched.width, batched.height)
    S.replay_setup(batched, pipe)
    pipe.finish()
    from puresoft3d_gb300.autotune import PINNED
    tune = autotune(pipe, lambda p: S.replay_frame(batched, p), "c4:%d:%dx%d" % (views, batched.width, batched.height),
                    args, PINNED["c4"] if views == 4096 else None)
    pipe.setFragmentCounting(True)
    st0 = pipe.stats()
    S.replay_frame(batched, pipe)
    pipe.finish()
    st1 = pipe.stats()
    pipe.setFragmentCounting(False)
    frags = st1["fragments"] - st0["fragments"]
    pairs = st1["bin_pairs"] - st0["bin_pairs"]
    counts = {"pairs": pairs, "triangles": st1["triangles"] - st0["triangles"],
              "shaded": st1["shaded"] - st0["shaded"]}
    launches_per_frame = st1["kernel_launches"] - st0["kernel_launches"]

    pipe.profile(True)
    pipe.profileRead()
    prof_frames = 3
    for _ in range(prof_frames):
        pipe.scrubL2()
        S.replay_frame(batched, pipe)
        pipe.finish()
    prof = pipe.profileRead()
    pipe.profile(False)

    pipe.beginCommands()
    S.replay_frame(batched, pipe)
    cb = pipe.endCommands()
    for _ in range(max(3, args.warmup)):
        cb.submit()
    pipe.finish()
    K = frames_per_step(args)
    clocks = ClockSampler()
    clocks.start()
    frame_ms = []
    for _ in range(args.steps * K):  # a step is K atlas passes, each timed alone after an L2 scrub
        pipe.scrubL2()
        pipe.timerBegin()
        cb.submit()
        frame_ms.append(pipe.timerEnd())
    pipe.finish()
    clk = clocks.stop()
    total_ms = allreduce_max(sum(frame_ms))
    ips = aggregate(views * args.steps * K, total_ms / 1e3)

    host = torch.empty((batched.height, batched.width, 4), dtype=torch.uint8, pin_memory=True).numpy()
    for _ in range(2):
        cb.submit(upload_inputs=True)
        pipe.readColour(host)
    e2e_steps = max(3, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        pipe.scrubL2()
        cb.submit(upload_inputs=True)
        pipe.readColour(host)
    e2e_sync_s = allreduce_max(time.perf_counter() - t0)
    pipe2 = twin(batched, tune)
    host2 = torch.empty_like(torch.from_numpy(host)).pin_memory().numpy()
    e2e_s = allreduce_max(e2e_pipelined([pipe, pipe2], lambda p: S.replay_frame(batched, p), [host, host2],
                                        e2e_steps))
    pipe2.close()
    in_bytes = cb.input_bytes()
    cb.destroy()
    pipe.close()

    # plain: one pass per view, each frame copied to its own slot of a device array
    alone = PuresoftPipeline(size, size)
    S.replay_setup(plain, alone)
    out = torch.empty((views, size, size, 4), dtype=torch.uint8, device="cuda")
    base, stride = out.data_ptr(), size * size * 4

    def plain_frame():
        for v in range(views):
            S.replay_ops(plain.info["view_frames"][v], alone)
            alone.readColourDevice(base + v * stride)

    tune_plain = autotune(alone, lambda p: [S.replay_ops(plain.info["view_frames"][v], p) for v in range(256)],
                          "c4plain:256:%d" % size, args)
    plain_frame()
    alone.finish()
    st0 = alone.stats()
    alone.scrubL2()
    alone.timerBegin()
    plain_frame()
    plain_ms = alone.timerEnd()
    plain_launches = alone.stats()["kernel_launches"] - st0["kernel_launches"]
    alone.beginCommands()
    plain_frame()
    pcb = alone.endCommands()
    for _ in range(2):
        pcb.submit()
    alone.finish()
    pg_ms = []
    for _ in range(max(2, args.steps // 4)):
        alone.scrubL2()
        alone.timerBegin()
        pcb.submit()
        pg_ms.append(alone.timerEnd())
    pcb.destroy()
    alone.close()
    plain_ips = views / (plain_ms / 1e3)
    plain_graph_ips = views / (statistics.median(pg_ms) / 1e3)

    roof = dominant_roofline(prof, prof_frames, batched, counts, tune["bin_width"],
                             KERNEL_TRAFFIC.get("c4", {}) if views == 4096 else {})
    line = {
        "metric": "images/s", "value": round(ips, 2), "unit": "images/s", "n_gpus": WORLD,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded meshes, cameras and textures per view)",
        "config": {"workload": CONFIGS["c4"]["desc"], "views": views, "view_size": size,
                   "atlas": [batched.width, batched.height], "triangles": batched.triangles(),
                   "frames_per_step": K,
                   "l2": "256 MB scrub before each timed step",
                   "parallelism": "replicas" if WORLD > 1 else "single GPU", "schedule": tune},
        "plain_images_per_s": {"immediate": round(plain_ips, 2), "graph": round(plain_graph_ips, 2),
                               "launches_per_view": round(plain_launches / views, 2), "schedule": tune_plain},
        "batched_over_plain": {"immediate": round(ips / WORLD / plain_ips, 2),
                               "graph": round(ips / WORLD / plain_graph_ips, 2)},
        "gfrag_per_s": round(frags * ips / views / 1e9, 4),
        "gshaded_per_s": round(counts["shaded"] * ips / views / 1e9, 4),
        "fragments_per_step": frags,
        "shaded_per_step": counts["shaded"],
        "gpu_launches": launches_per_frame * args.steps * K,
        "e2e": {"value": round(WORLD * views * e2e_steps / e2e_s, 2), "unit": "images/s",
                "mode": "steps back to back on two pipelines (double-buffered): each uploads its inputs and "
                        "copies its atlas to pinned host memory",
                "one_at_a_time": round(WORLD * views * e2e_steps / e2e_sync_s, 2),
                "h2d_bytes_per_step": in_bytes, "d2h_bytes_per_step": batched.width * batched.height * 4},
        "roofline": roof,
        "kernel_ms_per_step": {k: round(prof[k][1] / prof_frames, 5) for k in KERNELS if prof[k][0]},
        "clocks": clk,
    }
    if RANK == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_views(budget_s=args.cpu_budget)
    return line


def run_c5(args):
    """Config 5: the request loop with continuous batching against the
    one-request-at-a-time plain loop, on the same seeded job stream: closed
    loop (all jobs queued at t=0: capacity) and open loop (Poisson arrivals
    at 80 % of each arm's capacity: latency under load)."""
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.serving import PlainLoop, RenderServer, summarize
    pool = S.scene_c5_pool()
    base = S.c5_jobs(pool, n=args.jobs, rate=1.0)
    bw = args.bin_width or 16
    srv = RenderServer(pool, atlas=(4096, 4096), slots=2, bin_width=bw)
    plain = PlainLoop(pool, bin_width=bw)
    warm = base[:64]
    srv.serve(warm, realtime=False)
    plain.serve(warm, realtime=False)

    def at_rate(rate):
        return [dataclasses.replace(j, arrival=j.arrival / rate) for j in base]

    clocks = ClockSampler()
    clocks.start()
    up0 = sum(p.stats()["upload_bytes"] for p in srv.pipes)
    kl0 = sum(p.stats()["kernel_launches"] for p in srv.pipes)
    cap_b = summarize(srv.serve(base, realtime=False), realtime=False)
    h2d = (sum(p.stats()["upload_bytes"] for p in srv.pipes) - up0) / len(base)
    launches_b = sum(p.stats()["kernel_launches"] for p in srv.pipes) - kl0
    cap_p = summarize(plain.serve(base, realtime=False), realtime=False)
    loads = {}
    for name, cap in (("batched_capacity", cap_b["images_per_s"]), ("plain_capacity", cap_p["images_per_s"])):
        rate = 0.8 * cap
        jobs = at_rate(rate)
        loads[name] = {"rate_jobs_per_s": round(rate, 1),
                       "batched": {k: round(v, 3) for k, v in summarize(srv.serve(jobs)).items()},
                       "plain": {k: round(v, 3) for k, v in summarize(plain.serve(jobs)).items()}}
    clk = clocks.stop()
    d2h = sum(j.width * j.height * 4 for j in base) / len(base)
    cpu = cpu_baseline_jobs(budget_s=args.cpu_budget, pool=pool, jobs=base) if (
        RANK == 0 and not args.no_cpu_baseline) else None
    line = {
        "metric": "images/s", "value": round(cap_b["images_per_s"], 2), "unit": "images/s", "n_gpus": WORLD,
        "steps": len(base), "warmup": len(warm), "ms_per_step": round(1e3 / cap_b["images_per_s"], 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded job stream over a seeded resident pool)",
        "config": {"workload": CONFIGS["c5"]["desc"], "jobs": len(base), "bin_width": bw,
                   "pool_triangles": sum(pool.info["mesh_triangles"]),
                   "l2": "inputs (9.7M resident triangles, 1.2 GB of vertices) exceed L2",
                   "parallelism": "replicas" if WORLD > 1 else "single GPU"},
        "closed_loop": {"batched": {k: round(v, 3) for k, v in cap_b.items()},
                        "plain": {k: round(v, 3) for k, v in cap_p.items()}},
        "open_loop": loads,
        "batched_over_plain": round(cap_b["images_per_s"] / cap_p["images_per_s"], 2),
        "gpu_launches": int(launches_b),
        "e2e": {"value": round(cap_b["images_per_s"], 2), "unit": "images/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "note": "the serving loop is end to end: jobs enter from the host, images land in pinned host memory"},
        "roofline": None,
        "clocks": clk,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    srv.close()
    plain.close()
    return line


def cpu_baseline_views(budget_s=15.0, threads=None, sample_views=256, kind="auto"):
    """Config 4 on the host cores: the reference pipeline (or its oracle
    port) rendering the first views of the same seeded set one at a time in a
    128x128 pipeline."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from puresoft3d_gb300 import scenes as S
    from cpu_backends import OraclePipeline, RefPipeline
    threads = threads or os.cpu_count() or 1
    _, plain = S.scene_c4(views=sample_views)
    size = plain.info["view_size"]
    use_ref = _use_ref(kind)
    if use_ref:
        os.environ["PS3D_REF_THREADS"] = str(threads)
        pipe, kind = RefPipeline(size, size, threads), "reference"
    else:
        pipe, kind = OraclePipeline(size, size, threads), "port"
    S.replay_setup(plain, pipe)
    S.replay_ops(plain.info["view_frames"][0], pipe)
    n, t0 = 0, time.perf_counter()
    while True:
        S.replay_ops(plain.info["view_frames"][n % sample_views], pipe)
        pipe.readColour()
        n += 1
        el = time.perf_counter() - t0
        if el >= budget_s or n >= 20 * sample_views:
            break
    pipe.close()
    return {"value": round(n / el, 3), "unit": "images/s", "cores": threads, "kind": kind,
            "sample": "%d views (of the first %d of the seeded set) in %.1f s" % (n, sample_views, el)}


def run_frames_only(args):
    """For profilers: set up, then render --ncu-frames frames through the
    immediate path (no graph, no extra runs) and exit."""
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline
    scene = make_scene(args.config, args.views)
    pipe = PuresoftPipeline(scene.width, scene.height)
    S.replay_setup(scene, pipe)
    from puresoft3d_gb300.autotune import PINNED, apply
    if args.bin_width:
        apply(pipe, _flag_schedule(args))
    elif args.config in PINNED:
        apply(pipe, PINNED[args.config])
    for _ in range(args.ncu_frames):
        S.replay_frame(scene, pipe)
        pipe.finish()
    pipe.close()


def algorithmic_bytes(scene, counts):
    """Algorithmic bytes of the raster kernel per frame and per launch: what
    its work must move at least once -- the depth target's write (every pass
    here clears depth, fused into the raster), each triangle record once
    (64 B), each (bin, triangle) index once (4 B), one shade-list entry per
    covered pixel (8 B) and the clear colour of every uncovered pixel (4 B)."""
    info = scene.info
    w, h = scene.width, scene.height
    depth = w * h * 4
    launches = 1
    if scene.name == "c2":
        ss = info["shadow_size"]
        depth += ss * ss * 4
        launches = 2
    colour = counts["shaded"] * 8 + max(w * h - counts["shaded"], 0) * 4
    per_frame = depth + colour + counts["triangles"] * 64 + counts["pairs"] * 4
    return {"raster_per_frame": per_frame, "raster_launches_per_frame": launches}


def _targets(scene):
    """(width, height) of each pass's target in a frame of `scene`."""
    t = [(scene.width, scene.height)]
    if scene.name == "c2":
        t.append((scene.info["shadow_size"], scene.info["shadow_size"]))
    return t


def _radix_passes(w, h, bin_w):
    """The bin sort's LSD passes for one target: 8 bits of bin index each."""
    bins = -(-w // bin_w) * -(-h // 32)
    return ((bins - 1).bit_length() + 7) // 8 if bins > 1 else 0


def kernel_bytes_per_frame(kind, scene, counts, bin_w):
    """Algorithmic bytes per frame of each timed kernel class -- what its work
    must move at least once: raster as in algorithmic_bytes; the set-up reads
    each triangle's three positions (48 B) and writes its record (64 B) and
    its (bin, triangle) pairs (8 B each); each radix pass reads and writes
    every pair (16 B); the bin bounds write each bin's start and work item
    (8 B); the shade reads a shade-list entry and writes a pixel (12 B)."""
    if kind == "raster":
        return algorithmic_bytes(scene, counts)["raster_per_frame"]
    if kind == "setup":
        return counts["triangles"] * (48 + 64) + counts["pairs"] * 8
    if kind == "sort":
        passes = max(_radix_passes(w, h, bin_w) for w, h in _targets(scene))
        return counts["pairs"] * 16 * passes
    if kind == "bounds":
        return sum(-(-w // bin_w) * -(-h // 32) * 8 for w, h in _targets(scene))
    if kind == "shade":
        return counts["shaded"] * 12
    return None


def dominant_roofline(prof, prof_frames, scene, counts, bin_w, traffic):
    """The roofline object for the kernel class with the largest event-timed
    share: achieved = its algorithmic bytes per launch / its mean launch
    time, against the measured HBM copy bandwidth; traffic = the captured
    DRAM bytes per launch of that class (`traffic`: class -> bytes), when
    captured."""
    dom = max(prof, key=lambda k: prof[k][1])
    n_launch, ms = prof[dom]
    avg_ms = ms / max(n_launch, 1)
    peak, peak_kind = peaks()
    per_frame = kernel_bytes_per_frame(dom, scene, counts, bin_w)
    bytes_per_launch = per_frame / (n_launch / prof_frames) if per_frame and n_launch else None
    achieved = bytes_per_launch / (avg_ms / 1e3) / 1e9 if bytes_per_launch else None
    return {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 2) if achieved else None,
            "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 5) if achieved else None,
            "peak_source": peak_kind, "avg_launch_ms": round(avg_ms, 5),
            "bytes_per_launch": round(bytes_per_launch) if bytes_per_launch else None,
            "traffic": traffic.get(dom)}


def run_ours(args):
    from puresoft3d_gb300 import scenes as S
    from puresoft3d_gb300.pipeline import PuresoftPipeline, KERNELS
    scene = make_scene(args.config)
    pipe = PuresoftPipeline(scene.width, scene.height)
    S.replay_setup(scene, pipe)
    pipe.finish()
    from puresoft3d_gb300.autotune import PINNED
    tune = autotune(pipe, lambda p: S.replay_frame(scene, p), "%s:%dx%d:%d" % (
        args.config, scene.width, scene.height, scene.triangles()), args, PINNED.get(args.config))

    # fragments and pairs per frame (counting run, untimed)
    pipe.setFragmentCounting(True)
    st0 = pipe.stats()
    S.replay_frame(scene, pipe)
    pipe.finish()
    st1 = pipe.stats()
    pipe.setFragmentCounting(False)
    frags = st1["fragments"] - st0["fragments"]
    pairs = st1["bin_pairs"] - st0["bin_pairs"]
    counts = {"pairs": pairs, "triangles": st1["triangles"] - st0["triangles"],
              "shaded": st1["shaded"] - st0["shaded"]}
    launches_per_frame = st1["kernel_launches"] - st0["kernel_launches"]

    # per-kernel event timing over the non-graph path (untimed for value)
    pipe.profile(True)
    pipe.profileRead()
    prof_frames = max(3, min(args.steps, 10))
    for _ in range(prof_frames):
        pipe.scrubL2()
        S.replay_frame(scene, pipe)
        pipe.finish()
    prof = pipe.profileRead()
    pipe.profile(False)

    # recorded frame, replayed as a CUDA graph
    pipe.beginCommands()
    S.replay_frame(scene, pipe)
    cb = pipe.endCommands()
    for _ in range(max(3, args.warmup)):
        cb.submit()
    pipe.finish()

    K = frames_per_step(args)
    barrier()
    clocks = ClockSampler()
    clocks.start()
    frame_ms = []
    for _ in range(args.steps * K):  # a step is K frames, each timed alone after an L2 scrub
        pipe.scrubL2()
        pipe.timerBegin()
        cb.submit()
        frame_ms.append(pipe.timerEnd())
    pipe.finish()
    clk = clocks.stop()
    total_ms = allreduce_max(sum(frame_ms))

    # e2e through the public API with host buffers
    try:
        import torch
        host = torch.empty((scene.height, scene.width, 4), dtype=torch.uint8, pin_memory=True).numpy()
    except Exception:
        host = np.empty((scene.height, scene.width, 4), dtype=np.uint8)
    for _ in range(2):
        cb.submit(upload_inputs=True)
        pipe.readColour(host)
    t0 = time.perf_counter()
    for _ in range(args.steps * K):
        pipe.scrubL2()
        cb.submit(upload_inputs=True)
        pipe.readColour(host)
    e2e_sync_s = time.perf_counter() - t0
    pipe2 = twin(scene, tune)
    try:
        import torch
        host2 = torch.empty((scene.height, scene.width, 4), dtype=torch.uint8, pin_memory=True).numpy()
    except Exception:
        host2 = np.empty((scene.height, scene.width, 4), dtype=np.uint8)
    e2e_s = e2e_pipelined([pipe, pipe2], lambda p: S.replay_frame(scene, p), [host, host2], args.steps * K)
    pipe2.close()

    fps = aggregate(args.steps * K, total_ms / 1e3)
    fps_e2e = aggregate(args.steps * K, e2e_s)
    roof = dominant_roofline(prof, prof_frames, scene, counts, tune["bin_width"], KERNEL_TRAFFIC.get(args.config, {}))
    line = {
        "metric": "frames/s", "value": round(fps, 3), "unit": "frames/s", "n_gpus": WORLD,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded meshes and procedural textures)",
        "config": {"workload": CONFIGS[args.config]["desc"], "width": scene.width, "height": scene.height,
                   "triangles": scene.triangles(), "frames_per_step": K,
                   "l2": "256 MB scrub before each timed frame",
                   "parallelism": "replicas" if WORLD > 1 else "single GPU", "schedule": tune},
        "gfrag_per_s": round(frags * fps / WORLD / 1e9 * WORLD, 4),
        "gshaded_per_s": round(counts["shaded"] * fps / 1e9, 4),
        "fragments_per_frame": frags,
        "shaded_per_frame": counts["shaded"],
        "gpu_launches": launches_per_frame * args.steps * K,
        "e2e": {"value": round(fps_e2e, 3), "unit": "frames/s", "h2d_bytes_per_step": cb.input_bytes() * K,
                "d2h_bytes_per_step": scene.width * scene.height * 4 * K,
                "mode": "steps back to back on two pipelines (double-buffered): each uploads its inputs and "
                        "copies its frame to pinned host memory",
                "one_at_a_time": round(aggregate(args.steps * K, e2e_sync_s), 3)},
        "roofline": roof,
        "kernel_ms_per_frame": {k: round(prof[k][1] / prof_frames, 5) for k in KERNELS if prof[k][0]},
        "clocks": clk,
    }
    if RANK == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(scene, budget_s=args.cpu_budget)
        line["colour_error_vs_fp64"] = shading_error(scene)
    cb.destroy()
    pipe.close()
    return line


def shading_error(scene):
    """The frame's shaded fragments: FP32 pre-truncation colour against an
    FP64 re-shade of the same fragments, per channel in 8-bit units (from the
    oracle, whose colour the GPU matches bit for bit)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from puresoft3d_gb300 import scenes as S
    from cpu_backends import OraclePipeline
    o = OraclePipeline(scene.width, scene.height, os.cpu_count() or 1)
    o.measureColourError()
    S.replay_setup(scene, o)
    S.replay_frame(scene, o)
    e = o.colourError()
    o.close()
    return {"max": round(e["max"], 6), "mean": round(e["mean"], 9), "channels": e["channels"],
            "channels_off_by_1_or_more": e["over_1"]}


def _use_ref(kind):
    """Whether a CPU timing runs the reference build (kind "reference", or
    "auto" where it compiled on this host) or the oracle port ("port")."""
    have = os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libps3dref.so")) and os.uname().machine == "x86_64"
    if kind == "reference" and not have:
        raise SystemExit("the reference build is not available on this host")
    return have if kind == "auto" else kind == "reference"


def cpu_baseline(scene, budget_s=15.0, threads=None, kind="auto"):
    """The reference pipeline's CPU path timed on this host's cores: the
    reference build where it compiled here, else the oracle port of it."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from puresoft3d_gb300 import scenes as S
    from cpu_backends import OraclePipeline, RefPipeline
    threads = threads or os.cpu_count() or 1
    use_ref = _use_ref(kind)
    if use_ref:
        os.environ["PS3D_REF_THREADS"] = str(threads)
        pipe = RefPipeline(scene.width, scene.height, threads)
        kind = "reference"
    else:
        pipe = OraclePipeline(scene.width, scene.height, threads)
        kind = "port"
    S.replay_setup(scene, pipe)
    S.replay_frame(scene, pipe)  # warm-up
    frames, t0 = 0, time.perf_counter()
    while True:
        S.replay_frame(scene, pipe)
        frames += 1
        el = time.perf_counter() - t0
        if el >= budget_s or frames >= 200:
            break
    pipe.close()
    return {"value": round(frames / el, 4), "unit": "frames/s", "cores": threads, "kind": kind,
            "sample": "%d frames of the same workload in %.1f s" % (frames, el)}


def cpu_baseline_jobs(budget_s=15.0, threads=None, pool=None, jobs=None, kind="auto"):
    """Config 5 on the host cores: the reference pipeline (or its oracle
    port) rendering the seeded jobs one at a time, one pipeline per
    resolution, for a bounded time."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from puresoft3d_gb300 import scenes as S
    from cpu_backends import OraclePipeline, RefPipeline
    threads = threads or os.cpu_count() or 1
    pool = pool or S.scene_c5_pool()
    jobs = jobs or S.c5_jobs(pool, n=2000, rate=1.0)
    use_ref = _use_ref(kind)
    if use_ref:
        os.environ["PS3D_REF_THREADS"] = str(threads)
    pipes = {}
    for wh in S.C5_RESOLUTIONS:
        p = RefPipeline(wh[0], wh[1], threads) if use_ref else OraclePipeline(wh[0], wh[1], threads)
        S.replay_setup(pool, p)
        pipes[wh] = p
    n, t0 = 0, time.perf_counter()
    while True:
        j = jobs[n % len(jobs)]
        p = pipes[(j.width, j.height)]
        S.replay_ops([("clearDepth", 1.0), ("clearColour", 0xFF000000)] + pool.info["common"] + j.ops, p)
        p.readColour()
        n += 1
        el = time.perf_counter() - t0
        if el >= budget_s or n >= len(jobs):
            break
    for p in pipes.values():
        p.close()
    return {"value": round(n / el, 3), "unit": "images/s", "cores": threads,
            "kind": "reference" if use_ref else "port", "jobs_done": n,
            "sample": "the first %d jobs of the seeded stream, one at a time, in %.1f s" % (n, el)}


def run_calibration(args):
    """The reference build against the oracle port on this host, same
    workload, same thread count: how fast the port (the CPU arm on hosts
    where the reference does not build) runs relative to the reference's own
    code.  x86-64 hosts with the reference build only."""
    threads = args.cpu_threads or os.cpu_count() or 1
    out = {"impl": "reference", "calibration": True, "config": {"workload": CONFIGS[args.config]["desc"]},
           "threads": threads, "host": os.uname().machine}
    jobs = None
    for kind in ("reference", "port"):
        if args.config == "c4":
            v = cpu_baseline_views(budget_s=args.cpu_budget, threads=threads, kind=kind)
        elif args.config == "c5":
            # the port renders exactly the jobs the reference finished in its budget
            from puresoft3d_gb300 import scenes as S
            pool = S.scene_c5_pool()
            jobs = jobs or S.c5_jobs(pool, n=2000, rate=1.0)
            v = cpu_baseline_jobs(budget_s=args.cpu_budget if kind == "reference" else 1e9, threads=threads,
                                  pool=pool, jobs=jobs, kind=kind)
            jobs = jobs[:v["jobs_done"]]
        else:
            v = cpu_baseline(make_scene(args.config), budget_s=args.cpu_budget, threads=threads, kind=kind)
        out[kind] = v
    out["port_over_reference"] = round(out["port"]["value"] / out["reference"]["value"], 3)
    return out


def run_reference(args):
    if args.calibrate:
        return run_calibration(args)
    if args.config == "c4":
        return run_reference_views(args)
    if args.config == "c5":
        v = cpu_baseline_jobs(budget_s=args.cpu_budget)
        return {"impl": "reference", "metric": "images/s", "value": v["value"], "unit": "images/s",
                "n_gpus": WORLD, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 / v["value"], 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": {"workload": CONFIGS["c5"]["desc"]}, "cpu_baseline": v,
                "e2e": {"value": v["value"], "unit": "images/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    scene = make_scene(args.config)
    per = max(2.0, args.cpu_budget / max(args.steps, 1))
    vals = []
    cb = None
    for _ in range(args.warmup):
        cpu_baseline(scene, budget_s=0.1)
    t0 = time.perf_counter()
    frames = 0
    for _ in range(args.steps):
        cb = cpu_baseline(scene, budget_s=per)
        vals.append(cb["value"])
        frames += int(cb["sample"].split()[0])
    el = time.perf_counter() - t0
    v = statistics.median(vals)
    K = frames_per_step(args)
    return {"impl": "reference", "metric": "frames/s", "value": v, "unit": "frames/s", "n_gpus": WORLD,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * K / v, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": CONFIGS[args.config]["desc"], "frames_per_step": K,
                       "note": "each step a bounded sample of the workload on the host cores"},
            "cpu_baseline": {"value": v, "unit": "frames/s", "cores": cb["cores"], "kind": cb["kind"],
                             "sample": "%d steps, %d frames in %.1f s" % (args.steps, frames, el)},
            "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_reference_views(args):
    per = max(2.0, args.cpu_budget / max(args.steps, 1))
    cpu_baseline_views(budget_s=0.1)
    vals, n_total, t0 = [], 0, time.perf_counter()
    cb = None
    for _ in range(args.steps):
        cb = cpu_baseline_views(budget_s=per)
        vals.append(cb["value"])
        n_total += int(cb["sample"].split()[0])
    el = time.perf_counter() - t0
    v = statistics.median(vals)
    K = frames_per_step(args)
    return {"impl": "reference", "metric": "images/s", "value": v, "unit": "images/s", "n_gpus": WORLD,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * 4096 * K / v, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": CONFIGS["c4"]["desc"], "frames_per_step": K},
            "cpu_baseline": {"value": v, "unit": "images/s", "cores": cb["cores"], "kind": cb["kind"],
                             "sample": "%d steps, %d views in %.1f s" % (args.steps, n_total, el)},
            "e2e": {"value": v, "unit": "images/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


_pg = None


def init_dist():
    global _pg
    if WORLD > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        _pg = dist


def barrier():
    if _pg:
        _pg.barrier()


def allreduce_max(x):
    if not _pg:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    _pg.all_reduce(t, op=_pg.ReduceOp.MAX)
    return float(t.item())


def aggregate(units_per_rank, seconds):
    """Whole-job throughput of the replicas: every rank processed
    units_per_rank units; the job took as long as the slowest rank."""
    return WORLD * units_per_rank / allreduce_max(seconds)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--config", default="c2", choices=sorted(CONFIGS))
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--cpu-threads", type=int, default=0, help="CPU timings: threads (default: every host core)")
    ap.add_argument("--frames-per-step", type=int, default=0,
                    help="frames (c4: atlas passes) per timed step (default: per workload, FRAMES_PER_STEP)")
    ap.add_argument("--calibrate", action="store_true",
                    help="with --impl reference: time the reference build and the oracle port side by side")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ncu-frames", type=int, default=0, help="render N frames for a profiler and exit")
    ap.add_argument("--views", type=int, default=4096, help="config 4: number of views")
    ap.add_argument("--jobs", type=int, default=2000, help="config 5: number of jobs")
    ap.add_argument("--bin-width", type=int, default=0, choices=[0, 8, 16, 32],
                    help="fix the schedule (with --raster-occupancy) instead of autotuning it")
    ap.add_argument("--raster-occupancy", type=int, default=0, choices=[0, 8])
    ap.add_argument("--span-culling", type=int, default=1, choices=[0, 1],
                    help="with --bin-width: raster variant with (1) or without (0) the span occlusion test")
    ap.add_argument("--row-split", type=int, default=1, choices=[1, 2, 4, 8],
                    help="with --bin-width: raster blocks per bin (crowded bins shared out by rows)")
    ap.add_argument("--warp-bins", type=int, default=0, choices=[0, 1],
                    help="with --bin-width 8 or 16: one raster warp per bin (1) or four sharing it (0)")
    ap.add_argument("--span-items", type=int, default=0, choices=[0, 1],
                    help="with --bin-width: bin short triangles' row spans as set-up items (1) or whole triangles (0)")
    ap.add_argument("--lazy-varyings", type=int, default=0, choices=[0, 1],
                    help="with --bin-width: the shade computes its winners' vertex varyings (1) or the set-up "
                         "stores them (0)")
    ap.add_argument("--autotune", action="store_true",
                    help="time every schedule candidate on the frame and use the fastest (default: the pinned one)")
    args = ap.parse_args()
    if args.ncu_frames:
        run_frames_only(args)
        return
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        if RANK != 0:
            return
        print(json.dumps(run_reference(args)), flush=True)
        return
    init_dist()
    line = {"c4": run_c4, "c5": run_c5}.get(args.config, run_ours)(args)
    if RANK == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
