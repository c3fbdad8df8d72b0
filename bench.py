"""Benchmark of the path-tracing hot path: Msamples/s on the full-frame
workload (1920x1080, 16 spp, depth 8, 64 instances of 81,920-triangle
displaced icospheres, 16 emissive quads, Nishita sky and sun, bloom +
histogram auto exposure + AgX).

A step is one frame: kpt_render_frame(16) -- sky constants, camera rays, the
path wave (shade / shadow / extension kernels per level), sky queue,
accumulation and the whole post chain in one CUDA graph.  `value` is W*H*spp per step over
the device time of K steps (CUDA events on the library's stream, scene and
buffers resident in HBM, L2 flushed between steps).  `e2e` is the same
metric through the public API with the display image read back to host
memory every step.  The roofline is that of the dominant ray kernel
(extension or shadow rays): algorithmic bytes (24 B per box test, 40 B per
triangle test, 64 B per instance transform, counted in-kernel) over its
device time (event nodes around each launch in the graph) against the
measured HBM copy bandwidth.

The same run times the reference's own CUDA megakernel on the same scene
(built unmodified for sm_103a with its fast maths from the staged reference
sources by oracle/build_ref.sh; `megakernel`, `vs_megakernel`) and, as
`cpu_baseline`, the reference's own code built for the host cores on a
bounded sample of the frame.

--impl reference times that host build of the reference on all host cores
(kind "reference"; the oracle port, kind "port", only where the staged
sources are absent), on bounded samples of the same frame.
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Msamples/s @1080p (full-frame plain method, 16 spp, depth 8)"
W, H, SPP, DEPTH = 1920, 1080, 16, 8
WORKLOAD = "icosphere_grid_1080p_16spp_depth8"


# Counters of the largest launch of each ray kernel from one ncu --set full
# capture of the current build on the 960x540x8 case
# (profiles/wave_kernels_960x540x8.md): SIMT efficiency (active threads per
# warp instruction / 32), issue-active fraction, cache hit rates, DRAM
# throughput against its peak, the top stall.
NCU_RAY_KERNELS = {
    "extend": {"simt_efficiency": 11.68 / 32, "issue_active": 0.693, "l1_hit": 0.686, "l2_hit": 0.825,
               "dram_throughput_of_peak": 0.0154, "alu_pipe_active": 0.534,
               "top_stall": "long scoreboard, 3.67 cycles per issue"},
    "shadow": {"simt_efficiency": 11.44 / 32, "issue_active": 0.710, "l1_hit": 0.674, "l2_hit": 0.817,
               "dram_throughput_of_peak": 0.0125, "alu_pipe_active": 0.528,
               "top_stall": "long scoreboard"},
}


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(x, world, device=None):
    """The largest x over the ranks of a replicas run (all-reduce MAX over the
    default process group); x itself with one rank.  Timings are reduced this
    way, so a run's time is its slowest replica's."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            return float(json.load(open(p))["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def full_scene():
    """The full-frame workload, its sky in the arithmetic of the reference's
    GPU build (kpt_settings.sky_arith = 1), the build whose megakernel it is
    compared with."""
    from kittlespt_gb300 import scenes as S
    sc = S.scene_full(W, H, SPP, DEPTH)
    sc.sky_arith = 1
    return sc


def cpu_renderer(scene):
    """The CPU implementation timed as the baseline: the reference's own
    path-tracing code built for the host cores (oracle/_ref/libkpt_ref_host.so,
    kind "reference") where its sources were staged and built, else the
    oracle, our FP32 restatement of it (kind "port").  Returns (scene handle,
    kind, note)."""
    from oracle import oracle as O
    if O.available("ref"):
        return O.Scene(scene, "ref"), "reference", "reference host build (oracle/_ref/libkpt_ref_host.so)"
    why = "staged reference sources absent" if not O.ref_staged() else "reference host build missing"
    return O.Scene(scene), "port", f"oracle port ({why})"


def cpu_sample_rate(scene, max_seconds=20.0, min_seconds=8.0):
    """The CPU baseline on all host cores, rendering bands of rows of the same
    frame at 1 spp until min_seconds of work; returns Msamples/s, cores, kind
    and a description of the sample."""
    cores = os.cpu_count() or 1
    sc, kind, note = cpu_renderer(scene)
    band = 8
    rows_done, t0 = 0, time.perf_counter()
    row = 0
    while True:
        sc.render_samples(sample0=0, nsamples=1, rng_order=0, row0=row, nrows=band, nthreads=cores,
                          want_radiance=False)
        rows_done += band
        row = (row + 67 * band) % (H - band)
        el = time.perf_counter() - t0
        if el >= min_seconds or el >= max_seconds:
            break
        if el < 1.0:
            band = min(band * 2, 256)
    samples = rows_done * W
    rate = samples / el / 1e6
    return rate, cores, kind, (f"{note}: {rows_done} rows x {W} px x 1 spp of the {W}x{H} frame "
                               f"({samples} samples, {el:.1f} s)")


def megakernel_rate(scene, device, frames=SPP, warmup=2):
    """The reference's own CUDA megakernel (computePathTraceSamplesMegaKernel,
    built unmodified for sm_103a with its fast maths by oracle/build_ref.sh
    gpu) on the same scene: `frames` frames of one sample each (frame index =
    sample index, as the reference accumulates), each timed with CUDA events
    around launchPathTraceComputeMegaKernel.  Msamples/s = W*H*frames over
    the summed kernel time.  Returns a dict, or one with "unavailable"."""
    from oracle import oracle as O
    if not O.available("refgpu"):
        return {"unavailable": "reference GPU build absent (sources not staged)"}
    t0 = time.perf_counter()
    try:
        g = O.RefGpuScene(scene, device)
    except RuntimeError as e:   # a tree too deep for its 16-entry stacks: nothing was launched
        return {"unavailable": f"megakernel not run: {e}"}
    build_s = time.perf_counter() - t0
    try:
        depth = g.tree_depth()
        g.render(0, warmup, clear=True, want_accum=False)
        with ClockSampler(device) as clk:
            time.sleep(0.5)
            _, ms = g.render(0, frames, clear=True, want_accum=False)
        total = float(np.sum(ms))
    finally:
        g.close()
    return {"value": W * H * frames / (total / 1e3) / 1e6, "unit": "Msamples/s", "frames": frames,
            "spp_per_frame": 1, "ms_per_frame": total / frames, "kernel": "computePathTraceSamplesMegaKernel",
            "build": "reference shaders/*.cu unmodified, one translation unit, nvcc -use_fast_math sm_103a",
            "timing": "CUDA events around each launchPathTraceComputeMegaKernel (8x8 blocks)",
            "tree_depth": depth, "scene_build_s": build_s, "clocks": clk.summary()}


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return
    scene = full_scene()
    cores = os.cpu_count() or 1
    sc, kind, note = cpu_renderer(scene)
    band = 4
    # size one step to a few seconds
    t0 = time.perf_counter()
    sc.render_samples(0, 1, rng_order=0, row0=0, nrows=band, nthreads=cores, want_radiance=False)
    dt = max(time.perf_counter() - t0, 1e-3)
    band = int(min(max(band * 3.0 / dt, 4), H))
    for w in range(args.warmup):
        sc.render_samples(0, 1, rng_order=0, row0=(w * 97) % (H - band + 1), nrows=band, nthreads=cores,
                          want_radiance=False)
    t0 = time.perf_counter()
    for k in range(args.steps):
        sc.render_samples(0, 1, rng_order=0, row0=(k * 131) % (H - band + 1), nrows=band, nthreads=cores,
                          want_radiance=False)
    el = time.perf_counter() - t0
    samples = band * W * args.steps
    value = samples / el / 1e6
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Msamples/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded procedural scene, no reference dataset exists)",
           "config": config_of(scene, 1),
           "cpu_baseline": {"value": value, "unit": "Msamples/s", "cores": cores, "kind": kind,
                            "sample": f"{note}: per step {band} rows x {W} px x 1 spp of the {W}x{H} frame"},
           "e2e": {"value": value, "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def config_of(scene, world):
    return {"workload": WORKLOAD, "width": W, "height": H, "spp": SPP, "max_depth": DEPTH,
            "instances": len(scene.instances), "triangles_expanded": scene.ntris_expanded,
            "l2": "flushed between steps (256 MiB write)", "parallelism": "replicas" if world > 1 else "single"}


def run_gpu(args):
    import torch

    rank, world, local = env_rank()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from kittlespt_gb300 import build as B
    B.build()
    from kittlespt_gb300.renderer import Renderer
    from kittlespt_gb300 import _lib as K

    scene = full_scene()
    r = Renderer(local)
    r.initialize()
    r.load_scene(scene)
    stream = torch.cuda.ExternalStream(r.stream(), device=local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=local)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        r.execute_rendering(16.0, SPP)
        with torch.cuda.stream(stream):
            flush.add_(1.0)   # the first launch of a torch kernel loads its module: keep it out of the timed region
    r.synchronize()
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        # the sampler starts while one more untimed frame runs, so that its
        # start-up does not overlap the timed region
        r.execute_rendering(16.0, SPP)
        time.sleep(1.0)
        r.synchronize()
        st0 = r.stats()
        l0 = r.launch_count()
        barrier()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            start.record(stream)
            for k in range(args.steps):
                r.execute_rendering(16.0, SPP)
                if k + 1 < args.steps:
                    flush.add_(1.0)       # 256 MiB write between steps: L2 flush
            stop.record(stream)
        r.synchronize()
        torch.cuda.synchronize()
    barrier()
    ms = start.elapsed_time(stop)
    ms_max = max_over_ranks(ms, world, device=local)
    st1 = r.stats()
    launches = r.launch_count() - l0
    print(f"[bench] {args.steps} frames in {ms_max:.2f} ms ({ms_max / args.steps:.2f} ms/frame)", file=sys.stderr)
    # per-stage device times: event-record nodes between the launches of a few
    # more frames (their stages run one after another, so each is timed alone)
    n_timed = 3
    K.check(r._L.kpt_enable_timing(r.ctx, 1))
    for _ in range(n_timed + 1):
        r.execute_rendering(16.0, SPP)
    sms = (C.c_float * len(K.STAGES))()
    K.check(r._L.kpt_stage_ms(r.ctx, n_timed, sms))
    K.check(r._L.kpt_enable_timing(r.ctx, 0))
    stage_ms = {name: sms[i] / n_timed for i, name in enumerate(K.STAGES)}
    print("[bench] stage ms/frame (stages serialised): " + ", ".join(f"{k} {v:.2f}" for k, v in stage_ms.items()),
          file=sys.stderr)
    samples_step = W * H * SPP
    value = samples_step * args.steps * world / (ms_max / 1e3) / 1e6

    # roofline of the dominant ray kernel: algorithmic bytes per launch (24 B
    # per box test, 40 B per triangle test, 64 B per instance entered) over
    # its device time, from the event nodes around its launches
    def delta(field):
        return (getattr(st1, field) - getattr(st0, field)) / args.steps
    kern = {"extend": ("k_extend", "path"), "shadow": ("k_shadow", "shadow")}
    # DRAM bytes per frame of each ray kernel from one ncu capture of the
    # 960x540x8 case (profiles/wave_kernels_960x540x8.md), scaled by samples
    # (x8) to this workload
    traffic = {"extend": (249.1e6 + 20.1e6) * 8.0, "shadow": (128.8e6 + 0.9e6) * 8.0}
    dom = max(kern, key=lambda k: stage_ms[k])
    kname, pre = kern[dom]
    rays_frame = delta("camera_rays") + delta("path_rays") + delta("shadow_rays")
    boxes, tris, insts = delta(pre + "_box_tests"), delta(pre + "_tri_tests"), delta(pre + "_inst_xforms")
    alg_bytes = 24.0 * boxes + 40.0 * tris + 64.0 * insts
    launch_ms = stage_ms[dom]
    achieved = alg_bytes / (launch_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()

    # end to end through the public API, every step: camera from host memory
    # (2 matrices), render the frame, read the display image into pinned host
    # memory
    img = torch.empty((H, W, 4), dtype=torch.float32, pin_memory=True)
    img_ptr = C.cast(img.data_ptr(), C.POINTER(C.c_float))
    ip = np.ascontiguousarray(scene.camera.inv_proj.T, np.float32).reshape(-1)
    iv = np.ascontiguousarray(scene.camera.inv_view.T, np.float32).reshape(-1)
    n_e2e = max(2, args.steps // 2)
    r.synchronize()
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        K.check(r._L.kpt_set_camera_inverse(r.ctx, K.fptr(ip), K.fptr(iv)))
        r.execute_rendering(16.0, SPP)
        K.check(r._L.kpt_read_image(r.ctx, img_ptr))
    e2e_s = max_over_ranks((time.perf_counter() - t0) / n_e2e, world, device=local)
    e2e = samples_step * world / e2e_s / 1e6
    overflow = st1.overflows - st0.overflows
    r.shutdown()

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        rate, cores, kind, desc = cpu_sample_rate(scene)
        cpu = {"value": rate, "unit": "Msamples/s", "cores": cores, "kind": kind, "sample": desc}
    batch = None
    if rank == 0 and not args.no_batch:
        batch = batch_rate(3, 1)
        print(f"[bench] 32 mixed jobs: batched {batch['batched']['Msamples_per_s']:.0f} Msamples/s (graph branches "
              f"{batch['batched_branches']['Msamples_per_s']:.0f}), one by one "
              f"{batch['one_by_one']['Msamples_per_s']:.0f} ({batch['speedup']:.2f}x)", file=sys.stderr)
    adjoint = None
    if rank == 0 and not args.no_adjoint:
        adjoint = adjoint_rate(max(3, args.steps // 2), 2)
        print(f"[bench] adjoint {adjoint['value']:.1f} gradient evaluations/s "
              f"(sky check {adjoint.get('max_rel_err_sky', float('nan')):.2e})", file=sys.stderr)
    mega = None
    if rank == 0 and not args.no_megakernel:
        mega = megakernel_rate(scene, local)
        if "value" in mega:
            print(f"[bench] reference megakernel {mega['ms_per_frame']:.2f} ms per 1-spp frame, "
                  f"{mega['value']:.1f} Msamples/s", file=sys.stderr)
    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "Msamples/s", "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
               "scaling": "weak" if world > 1 else "weak", "vs_baseline": None, "dtype": "f32",
               "data": "synthetic (seeded procedural scene, no reference dataset exists)",
               "config": config_of(scene, world),
               "roofline": {"bound": "latency", "kernel": kname, "achieved": achieved, "peak": peak,
                            "unit": "GB/s", "frac": achieved / peak,
                            "frac_of": "measured HBM copy bandwidth, for the kernel's algorithmic bytes",
                            "traffic": traffic[dom],
                            "traffic_gbs": traffic[dom] / (launch_ms / 1e3) / 1e9,
                            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per frame, "
                                              "960x540x8 capture scaled x8 by samples "
                                              "(profiles/wave_kernels_960x540x8.md)",
                            "peak_kind": peak_kind,
                            "why": "latency and issue bound: DRAM at ~1.5% of its peak, the algorithmic "
                                   "bytes served 69% by L1 and 83% of the rest by L2; issue slots at 69% "
                                   "with 11.7 of 32 lanes active per instruction; long-scoreboard stalls "
                                   "on dependent node and triangle fetches",
                            "ncu": NCU_RAY_KERNELS[dom],
                            "algorithmic_bytes_per_frame": alg_bytes, "kernel_ms_per_frame": launch_ms,
                            "launches_per_frame": DEPTH + (1 if dom == "shadow" else 0),
                            "kernel_ms_source": "event-record nodes around each launch in the frame graph "
                                                "(3 frames with the stages serialised)",
                            "box_tests": boxes, "tri_tests": tris, "inst_xforms": insts},
               "stage_ms_per_frame": stage_ms,
               "rays_per_s": rays_frame * args.steps * world / (ms_max / 1e3),
               "rays_per_frame": {"camera": delta("camera_rays"), "extension": delta("path_rays"),
                                  "shadow": delta("shadow_rays")},
               "traversal_work_per_frame": {k: {"box_tests": delta(pre + "_box_tests"),
                                                "tri_tests": delta(pre + "_tri_tests"),
                                                "inst_xforms": delta(pre + "_inst_xforms")}
                                            for k, pre in (("extension", "path"), ("shadow", "shadow"))},
               "cpu_baseline": cpu,
               "adjoint": adjoint,
               "batch": batch,
               "megakernel": mega,
               "megakernel_msamples_s": mega.get("value") if mega else None,
               "vs_megakernel": value / world / mega["value"] if mega and "value" in mega else None,
               "e2e": {"value": e2e, "unit": "Msamples/s", "h2d_bytes_per_step": 128,
                       "d2h_bytes_per_step": W * H * 16},
               "gpu_launches": int(launches), "traversal_overflows": int(overflow),
               "clocks": clk.summary()}
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


BATCH_JOBS = 32
BATCH_RES = [(128, 128), (256, 256), (512, 288), (1024, 1024), (1920, 1080)]


def batch_jobs(seed=4):
    """The mixed-job workload: 32 jobs in a seeded arrival order, resolution
    from BATCH_RES, spp U{1..16}, depth U{3..8}, scene from the small (sphere)
    or the full-frame (icosphere grid) family with U{1..64} object instances."""
    import dataclasses
    from kittlespt_gb300 import scenes as S
    rng = np.random.Generator(np.random.PCG64(seed))
    base = S.scene_full(W, H, SPP, DEPTH)
    objects, lights = base.instances[:64], base.instances[64:]
    jobs = []
    for _ in range(BATCH_JOBS):
        w, h = BATCH_RES[int(rng.integers(0, len(BATCH_RES)))]
        spp, depth = int(rng.integers(1, 17)), int(rng.integers(3, 9))
        n_inst = int(rng.integers(1, 65))
        if rng.integers(0, 2) == 0:
            sc = S.scene_small_n(w, h, spp, depth, n_inst, seed=int(rng.integers(0, 1 << 30)))
        else:
            sc = dataclasses.replace(base, instances=objects[:n_inst] + lights,
                                     camera=S.Camera.look_at((0.0, 4.0, 22.0), (0.0, 1.0, 0.0), 45.0, w, h),
                                     settings=S.settings(max_depth=depth, bloom=True, auto_exposure=True),
                                     width=w, height=h, spp=spp, name=f"icosphere_grid_{n_inst}")
        jobs.append(sc)
    return jobs


def batch_rate(steps, warmup):
    """Batched requests against the same jobs launched one by one: total
    Msamples/s and p50/p99 job latency (all jobs arrive at once; a job's
    latency is the wall time from the start of the round to the end of its
    frame, host submission included).  Returns a dict."""
    import torch
    from kittlespt_gb300 import build as B
    B.build()
    from kittlespt_gb300.renderer import Batch, Renderer
    jobs = batch_jobs()
    rs = []
    for sc in jobs:
        r = Renderer(0)
        r.initialize()
        r.load_scene(sc)
        rs.append(r)
    spp = [sc.spp for sc in jobs]
    samples = sum(sc.width * sc.height * sc.spp for sc in jobs)

    def one_by_one():
        lat, t0 = [], time.perf_counter()
        for r, s in zip(rs, spp):
            r.execute_rendering(16.0, s)
            r.synchronize()
            lat.append((time.perf_counter() - t0) * 1e3)
        return (time.perf_counter() - t0) * 1e3, np.array(lat)

    with Batch(0) as b:
        def batched(lanes):
            t0 = time.perf_counter()
            b.submit(rs, spp, lanes=lanes)
            t_sub = (time.perf_counter() - t0) * 1e3
            job_ms, _ = b.wait()
            return (time.perf_counter() - t0) * 1e3, job_ms + t_sub

        for _ in range(warmup):
            one_by_one()
            batched(0)
        t_tune = time.perf_counter()
        tuning, lanes, tuned_ms = b.autotune(rs, spp, reps=2)
        t_tune = time.perf_counter() - t_tune
        batched(lanes)   # instantiate the tuned graph outside the timed rounds
        seq = [one_by_one() for _ in range(steps)]
        bat = [batched(lanes) for _ in range(steps)]
        # the same batch with each job's frame a branch of the graph (no
        # queue spanning the jobs)
        b.shared = False
        batched(lanes)
        br = [batched(lanes) for _ in range(steps)]
        b.shared = True
    for r in rs:
        r.shutdown()
    torch.cuda.synchronize()
    seq_ms = float(np.mean([t for t, _ in seq]))
    bat_ms = float(np.mean([t for t, _ in bat]))
    br_ms = float(np.mean([t for t, _ in br]))
    seq_lat = np.concatenate([l for _, l in seq])
    bat_lat = np.concatenate([l for _, l in bat])
    br_lat = np.concatenate([l for _, l in br])
    return {"value": samples / bat_ms / 1e3, "unit": "Msamples/s", "ms_per_step": bat_ms,
           "config": {"workload": "batch_32_mixed_jobs", "jobs": BATCH_JOBS, "samples_per_round": samples,
                      "resolutions": [f"{sc.width}x{sc.height}" for sc in jobs], "spp": spp,
                      "depths": [int(sc.settings["max_depth"]) for sc in jobs],
                      "instances": [len(sc.instances) for sc in jobs]},
           "batched": {"Msamples_per_s": samples / bat_ms / 1e3, "round_ms": bat_ms,
                       "p50_latency_ms": float(np.percentile(bat_lat, 50)),
                       "p99_latency_ms": float(np.percentile(bat_lat, 99)),
                       "mode": "shared ray queues spanning the jobs"},
           "batched_branches": {"Msamples_per_s": samples / br_ms / 1e3, "round_ms": br_ms,
                                "p50_latency_ms": float(np.percentile(br_lat, 50)),
                                "p99_latency_ms": float(np.percentile(br_lat, 99)),
                                "mode": "each job's frame a branch of the graph"},
           "one_by_one": {"Msamples_per_s": samples / seq_ms / 1e3, "round_ms": seq_ms,
                          "p50_latency_ms": float(np.percentile(seq_lat, 50)),
                          "p99_latency_ms": float(np.percentile(seq_lat, 99))},
           "speedup": seq_ms / bat_ms,
           "autotune": {"tuning": tuning, "lanes": lanes, "device_ms": tuned_ms, "tuning_seconds": t_tune}}


def run_batch(args):
    """The batched-requests workload as its own bench line (--workload batch)."""
    b = batch_rate(args.steps, args.warmup)
    out = {"metric": "total Msamples/s, 32 mixed jobs (batched requests)", "value": b["value"],
           "unit": "Msamples/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": b["ms_per_step"], "higher_is_better": True, "dtype": "f32",
           "data": "synthetic (seeded mixed jobs of the small and full-frame scene families)"}
    out.update({k: v for k, v in b.items() if k not in ("value", "unit", "ms_per_step")})
    print(json.dumps(out))


ADJ_W, ADJ_H, ADJ_SPP, ADJ_DEPTH = 512, 512, 32, 6


def adjoint_scene(seed=7):
    """The differentiation workload: the sphere-pair scene at 512 x 512, depth
    6, materials with albedo U(0.1, 0.9)^3 and roughness U(0.05, 1), Rayleigh
    and Mie scale heights 8 km and 1.2 km."""
    from kittlespt_gb300 import scenes as S
    sc = S.scene_small(ADJ_W, ADJ_H, ADJ_SPP, ADJ_DEPTH)
    rng = np.random.Generator(np.random.PCG64(seed))
    mats = sc.materials.copy()
    for m in mats:
        m["albedo"] = rng.uniform(0.1, 0.9, 3)
        m["roughness"] = rng.uniform(0.05, 1.0)
    sc.materials = mats
    env = sc.env.copy()
    env["rayleigh_height"], env["mie_height"] = 8000.0, 1200.0
    sc.env = env
    return sc


def adjoint_rate(steps, warmup, check_sky=True):
    """Gradient evaluations per second of the L2 image loss on the
    differentiation workload: the split path-replay adjoint's forward half
    (one replay of 32 samples per pixel that keeps its records and gives the
    image), the loss's adjoint image, the backward half (the sweep of the
    records), all on the device (CUDA events on the library's stream), from
    an initial guess within +-20% of the parameters that rendered the target
    (target samples: seed 7, i.e.
    sample indices 7*32 .. 7*32+31).  With check_sky, the adjoint's
    derivatives for the six sky parameters -- which no sampling decision
    depends on -- are compared with central differences (h = 1e-2 relative)
    of the forward renderer's loss at the same point (max_rel_err_sky).  The
    single-precision renderer's differences for the weakest parameter
    (Rayleigh red) move by ~0.5% between h = 1e-3 and 1e-2 (measured: 8.9e-3
    and 2.4e-3 from the adjoint), so this check reads a few 1e-3; the
    adjoint's accuracy is checked against the FP64 oracle."""
    import torch
    from kittlespt_gb300 import build as B
    B.build()
    from kittlespt_gb300 import _lib as K
    from kittlespt_gb300.renderer import Renderer
    sc = adjoint_scene()
    r = Renderer(0)
    r.initialize()
    r.load_scene(sc)
    nmat = len(sc.materials)
    stream = torch.cuda.ExternalStream(r.stream(), device=0)
    buf = torch.zeros((ADJ_SPP, ADJ_H, ADJ_W, 4), dtype=torch.float32, device="cuda")
    n = C.c_int()
    K.check(r._L.kpt_adjoint_param_count(r.ctx, C.byref(n)))
    grad = torch.zeros(n.value, dtype=torch.float64, device="cuda")

    def apply(theta):
        for k, m in enumerate(sc.materials):
            mm = m.copy()
            mm["albedo"], mm["roughness"] = theta[4 * k:4 * k + 3], theta[4 * k + 3]
            r.set_material(k, mm)
        e = sc.env.copy()
        e["rayleigh"], e["mie"] = theta[-6:-3], theta[-3]
        e["rayleigh_height"], e["mie_height"] = theta[-2], theta[-1]
        r.set_procedural_environment_data(e)

    theta_true = []
    for m in sc.materials:
        theta_true += [float(x) for x in m["albedo"]] + [float(m["roughness"])]
    e = sc.env
    theta_true += [float(x) for x in e["rayleigh"]] + [float(e["mie"]), float(e["rayleigh_height"]),
                                                        float(e["mie_height"])]
    theta_true = np.array(theta_true)
    rng = np.random.Generator(np.random.PCG64(7))
    theta0 = theta_true * (1.0 + rng.uniform(-0.2, 0.2, theta_true.size))
    theta0[:4 * nmat] = np.clip(theta0[:4 * nmat], 0.02, 0.98)
    with torch.cuda.stream(stream):
        r.render_samples_device(7 * ADJ_SPP, ADJ_SPP, buf.data_ptr())
        target = buf.mean(dim=0).clone()
        apply(theta0)
        adj = torch.zeros((ADJ_H, ADJ_W, 4), dtype=torch.float32, device="cuda")
        img = torch.zeros((ADJ_H, ADJ_W, 4), dtype=torch.float32, device="cuda")

        def gradient():
            # the split adjoint: one replay that keeps its records and gives
            # the image, the loss's adjoint image, the sweep of the records
            r.adjoint_forward_device(0, ADJ_SPP, img.data_ptr())
            adj[..., :3] = 2.0 * (img[..., :3] - target[..., :3])
            r.adjoint_backward_device(adj.data_ptr(), grad.data_ptr())

        for _ in range(warmup):
            gradient()
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
        ev[0].record(stream)
        for _ in range(steps):
            gradient()
        ev[1].record(stream)
        r.adjoint_forward_device(0, ADJ_SPP, img.data_ptr())
        ev[2].record(stream)
        adj[..., :3] = 2.0 * (img[..., :3] - target[..., :3])
        ev[3].record(stream)
        r.adjoint_backward_device(adj.data_ptr(), grad.data_ptr())
        ev[4].record(stream)
        # the one-call adjoint (a second replay of the forward renderer's samples) for comparison
        g_one = torch.zeros_like(grad)
        K.check(r._L.kpt_adjoint_device(r.ctx, 0, ADJ_SPP, adj.data_ptr(), g_one.data_ptr(), None))
        ev[5].record(stream)
        torch.cuda.synchronize()
    ms = ev[0].elapsed_time(ev[1]) / steps
    fwd_ms, loss_ms, bwd_ms, one_ms = (ev[1].elapsed_time(ev[2]), ev[2].elapsed_time(ev[3]),
                                       ev[3].elapsed_time(ev[4]), ev[4].elapsed_time(ev[5]))
    loss = float(((img[..., :3].double() - target[..., :3].double()) ** 2).sum())
    g = grad.cpu().numpy()
    gone = g_one.cpu().numpy()
    out = {"value": 1e3 / ms, "unit": "gradient evaluations/s", "ms_per_gradient": ms,
           "forward_replay_ms": fwd_ms, "loss_ms": loss_ms, "backward_ms": bwd_ms,
           "one_call_adjoint_ms": one_ms,
           "split_vs_one_call_max_rel_diff": float(np.max(np.abs(g - gone) / np.maximum(np.abs(gone), 1e-300))),
           "parameters": int(n.value),
           "config": {"workload": "adjoint_sphere_pair_512_32spp_depth6", "width": ADJ_W, "height": ADJ_H,
                      "spp": ADJ_SPP, "max_depth": ADJ_DEPTH, "samples_per_gradient": ADJ_W * ADJ_H * ADJ_SPP},
           "Msamples_per_s_replayed": ADJ_W * ADJ_H * ADJ_SPP / fwd_ms / 1e3,
           "loss": loss, "grad_norm": float(np.linalg.norm(g * np.abs(theta0)))}
    if check_sky:
        def loss_at(theta):
            apply(theta)
            r.render_samples_device(0, ADJ_SPP, buf.data_ptr())
            r.synchronize()
            im = buf.mean(dim=0)[..., :3].double()
            return float(((im - target[..., :3].double()) ** 2).sum())
        errs = []
        for i in range(theta0.size - 6, theta0.size):
            h = 1e-2 * abs(theta0[i])
            tp, tm = theta0.copy(), theta0.copy()
            tp[i] += h
            tm[i] -= h
            fd = (loss_at(tp) - loss_at(tm)) / (2.0 * h)
            errs.append(abs(g[i] - fd) / max(abs(fd), 1e-30))
        apply(theta0)
        out["max_rel_err_sky"] = float(max(errs))
        out["rel_err_sky"] = [float(x) for x in errs]
        out["accuracy_check"] = ("sky parameters against central differences (h = 1e-2) of the "
                                 "single-precision forward renderer's loss at this workload, whose "
                                 "Rayleigh-red difference itself moves by ~0.5% with h; all 18 parameters "
                                 "are checked against central differences (h = 1e-3) of the FP64 oracle to "
                                 "1e-3 in tests/test_adjoint.py")
    r.shutdown()
    return out


def run_adjoint(args):
    """The differentiation workload as its own bench line (--workload adjoint)."""
    a = adjoint_rate(args.steps, args.warmup)
    out = {"metric": "adjoint gradient evaluations/s (L2 image loss, 512x512, 32 spp, depth 6)",
           "value": a["value"], "unit": "gradients/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": a["ms_per_gradient"], "higher_is_better": True, "dtype": "f32",
           "data": "synthetic (seeded sphere-pair scene with random materials)",
           "config": dict(a["config"], parameters=a["parameters"]),
           "forward_replay_ms": a["forward_replay_ms"], "loss_ms": a["loss_ms"], "backward_ms": a["backward_ms"],
           "one_call_adjoint_ms": a["one_call_adjoint_ms"],
           "split_vs_one_call_max_rel_diff": a["split_vs_one_call_max_rel_diff"],
           "Msamples_per_s_replayed": a["Msamples_per_s_replayed"], "loss": a["loss"], "grad_norm": a["grad_norm"],
           "max_rel_err_sky": a.get("max_rel_err_sky"), "accuracy_check": a.get("accuracy_check")}
    print(json.dumps(out))


def run_traversal(args):
    """Traversal stress: one BLAS of 2,000,000 random triangles, 1,048,576
    incoherent rays from the bounding sphere plus 4 diffuse bounces
    (kpt_trace_bounces_device); rays/s over the rays actually traced (a chain
    stops at its first miss)."""
    import torch
    from kittlespt_gb300 import build as B
    B.build()
    from kittlespt_gb300 import scenes as S
    from kittlespt_gb300.renderer import Renderer
    sc = S.scene_traversal(2_000_000)
    o, d = S.random_rays(1_048_576)
    n, nb = o.shape[0], 4
    r = Renderer(0)
    r.initialize()
    r.load_scene(sc)
    stream = torch.cuda.ExternalStream(r.stream(), device=0)
    to = torch.from_numpy(np.ascontiguousarray(o, np.float32)).cuda()
    td = torch.from_numpy(np.ascontiguousarray(d, np.float32)).cuda()
    inst = torch.empty((nb + 1) * n, dtype=torch.int32, device="cuda")
    tri = torch.empty_like(inst)
    t = torch.empty((nb + 1) * n, dtype=torch.float32, device="cuda")

    def step():
        r.trace_bounces_device(n, to.data_ptr(), td.data_ptr(), nb, inst.data_ptr(), tri.data_ptr(), t.data_ptr())
    for _ in range(args.warmup):
        step()
    r.synchronize()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    with torch.cuda.stream(stream):
        ev[0].record(stream)
        for _ in range(args.steps):
            step()
        ev[1].record(stream)
    r.synchronize()
    torch.cuda.synchronize()
    ms = ev[0].elapsed_time(ev[1]) / args.steps
    hits = inst.view(nb + 1, n).cpu().numpy() >= 0
    traced = n + int(hits[:-1].sum())
    r.shutdown()
    out = {"metric": "rays/s, traversal stress (2M random triangles, 1M rays + 4 diffuse bounces)",
           "value": traced / (ms / 1e3), "unit": "rays/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": ms, "higher_is_better": True, "dtype": "f32",
           "data": "synthetic (seeded random triangles and rays)",
           "config": {"workload": "random_triangles_2M_rays_1M_bounces_4", "triangles": 2_000_000, "rays": n,
                      "bounces": nb, "rays_traced_per_step": traced}}
    print(json.dumps(out))


def run_blas(args):
    """BLAS build time on upload (kpt_upload_mesh), host build against the
    device build (kpt_set_blas_build), for the 2M-random-triangle mesh and
    one 81,920-triangle displaced icosphere of the full-frame scene.  The
    device time includes the positions' copy to the GPU and the tree's copy
    back; both builds give the same tree (tests/test_blas_build.py)."""
    from kittlespt_gb300 import _lib as K
    from kittlespt_gb300 import scenes as S
    L = K.load()
    ctx = C.c_void_p()
    K.check(L.kpt_create(0, C.byref(ctx)))
    meshes = [("random_triangles_2M", S.random_triangles(2_000_000, seed=3)),
              ("displaced_icosphere_81920", S.displaced_icosphere(subdiv=6, amplitude=0.1, seed=0))]
    res = {}
    try:
        for name, m in meshes:
            pos = np.ascontiguousarray(m.positions, np.float32).reshape(-1)
            n = m.ntris
            mat = np.zeros(n, np.int32)
            out = C.c_int()
            times = {}
            for device, reps in ((0, 1), (1, max(1, args.steps))):
                K.check(L.kpt_set_blas_build(ctx, device))
                for _ in range(args.warmup if device else 0):
                    K.check(L.kpt_upload_mesh(ctx, n, K.fptr(pos), None, None, K.iptr(mat), C.byref(out)))
                    K.check(L.kpt_clear_scene(ctx))
                best = float("inf")
                for _ in range(reps):
                    t0 = time.perf_counter()
                    K.check(L.kpt_upload_mesh(ctx, n, K.fptr(pos), None, None, K.iptr(mat), C.byref(out)))
                    best = min(best, time.perf_counter() - t0)
                    K.check(L.kpt_clear_scene(ctx))
                times["device" if device else "host"] = best * 1e3
            # refit (kpt_refit_mesh) of the same mesh in a committed scene,
            # positions scaled by 1.1
            K.check(L.kpt_set_blas_build(ctx, 1))
            mats = (K.Material * 1)()
            mats[0].albedo[:] = (0.5, 0.5, 0.5)
            mats[0].roughness, mats[0].ior, mats[0].normal_scale = 0.5, 1.5, 1.0
            mats[0].albedo_tex = mats[0].orm_tex = mats[0].transmission_tex = mats[0].emission_tex = -1
            mats[0].normal_tex = -1
            K.check(L.kpt_set_materials(ctx, 1, mats))
            K.check(L.kpt_upload_mesh(ctx, n, K.fptr(pos), None, None, K.iptr(mat), C.byref(out)))
            ident = np.eye(4, dtype=np.float32).reshape(-1)
            inst = C.c_int()
            K.check(L.kpt_add_instance(ctx, out.value, K.fptr(ident), -1, C.byref(inst)))
            K.check(L.kpt_commit_scene(ctx))
            moved = np.ascontiguousarray(pos * np.float32(1.1), np.float32)
            refit = float("inf")
            for _ in range(max(2, args.steps)):
                t0 = time.perf_counter()
                K.check(L.kpt_refit_mesh(ctx, out.value, K.fptr(moved), None))
                refit = min(refit, time.perf_counter() - t0)
            K.check(L.kpt_clear_scene(ctx))
            res[name] = {"triangles": n, "host_ms": times["host"], "device_ms": times["device"],
                         "speedup": times["host"] / times["device"], "refit_ms": refit * 1e3}
            print(f"[bench] {name}: host {times['host']:.1f} ms, device {times['device']:.1f} ms, "
                  f"refit {refit * 1e3:.1f} ms", file=sys.stderr)
    finally:
        L.kpt_destroy(ctx)
    big = res["random_triangles_2M"]
    out = {"metric": "BLAS build, Mtriangles/s (kpt_upload_mesh with the device build, 2M random triangles)",
           "value": big["triangles"] / big["device_ms"] / 1e3, "unit": "Mtriangles/s", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": big["device_ms"], "higher_is_better": True,
           "dtype": "f32", "data": "synthetic (seeded random triangles, displaced icosphere)",
           "config": {"workload": "blas_build"}, "builds": res}
    print(json.dumps(out))


def run_upscale(args):
    """Upscaling (kpt_settings.upscale): the full-frame scene displayed at
    1920x1080 and rendered at 768x432 (output / 2.5), 16 spp, depth 8, the
    render upscaled bilinearly (1) or by the FSR path, EASU + RCAS (2), with
    bloom, exposure and tonemapping at the output size; native 1080p frames
    (0) beside them.  Device time per frame over K frames (CUDA events on the
    library's stream, L2 flushed between frames) and the post chain's own time
    (event nodes around it in the frame's graph)."""
    import torch
    from kittlespt_gb300 import _lib as K
    from kittlespt_gb300 import scenes as S
    from kittlespt_gb300.renderer import Renderer
    r = Renderer(0)
    r.initialize()
    r.load_scene(S.scene_full(W, H, SPP, DEPTH))
    stream = torch.cuda.ExternalStream(r.stream(), device=0)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=0)
    res = {}
    try:
        for mode, name in ((0, "native"), (1, "bilinear"), (2, "fsr")):
            r.set_renderer_settings(upscale=mode)
            for _ in range(args.warmup):
                r.execute_rendering(16.0, SPP)
                with torch.cuda.stream(stream):
                    flush.add_(1.0)
            r.synchronize()
            torch.cuda.synchronize()
            start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                start.record(stream)
                for k in range(args.steps):
                    r.execute_rendering(16.0, SPP)
                    if k + 1 < args.steps:
                        flush.add_(1.0)
                stop.record(stream)
            r.synchronize()
            torch.cuda.synchronize()
            ms = start.elapsed_time(stop) / args.steps
            K.check(r._L.kpt_enable_timing(r.ctx, 1))
            for _ in range(4):
                r.execute_rendering(16.0, SPP)
            sms = (C.c_float * len(K.STAGES))()
            K.check(r._L.kpt_stage_ms(r.ctx, 3, sms))
            K.check(r._L.kpt_enable_timing(r.ctx, 0))
            rw, rh = r.render_size()
            res[name] = {"render": f"{rw}x{rh}", "ms_per_frame": ms, "post_ms": sms[K.STAGES.index("post")] / 3}
            print(f"[bench] {name}: render {rw}x{rh}, {ms:.2f} ms/frame, post chain "
                  f"{res[name]['post_ms']:.3f} ms", file=sys.stderr)
    finally:
        r.shutdown()
    f = res["fsr"]
    out = {"metric": "frames/s, 1920x1080 output upscaled by FSR 1.0 from 768x432 (16 spp, depth 8)",
           "value": 1e3 / f["ms_per_frame"], "unit": "frames/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": f["ms_per_frame"], "higher_is_better": True, "dtype": "f32",
           "data": "synthetic (seeded procedural scene)",
           "config": {"workload": "upscale_1080p_from_768x432", "output": f"{W}x{H}", "spp": SPP,
                      "max_depth": DEPTH, "l2": "flushed between frames"}, "modes": res}
    print(json.dumps(out))


def run_temporal(args):
    """Temporal accumulation (kpt_settings.temporal_accumulation): the
    full-frame scene at 1920x1080, 16 spp per call (each sample one reference
    frame, blended into the reprojected history), the camera moving a little
    before every call; the same frames with the running mean beside them.
    Device time per call over K calls (CUDA events on the library's stream, L2
    flushed between calls).  The temporal blend in the reference GPU build's
    arithmetic (temporal_arith 1, the default: per-pixel matrix inverses and
    the visible surface recomputed) and in IEEE (0)."""
    import torch
    from kittlespt_gb300 import scenes as S
    from kittlespt_gb300.renderer import Renderer
    sc = S.scene_full(W, H, SPP, DEPTH)
    r = Renderer(0)
    r.initialize()
    r.load_scene(sc)
    stream = torch.cuda.ExternalStream(r.stream(), device=0)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=0)
    ip = sc.camera.inv_proj.astype(np.float32)
    res = {}
    try:
        for mode, arith, name in ((0, 0, "running_mean"), (1, 0, "temporal_ieee"), (1, 1, "temporal")):
            r.set_renderer_settings(temporal_accumulation=mode, temporal_arith=arith)
            k = 0

            def frame():
                nonlocal k
                iv = sc.camera.inv_view.astype(np.float32).copy()
                iv[:3, 3] += np.float32(0.02 * (k % 16))   # a slow pan, back every 16 frames
                r.set_camera_inverse(ip, iv)
                r.execute_rendering(16.0, SPP)
                k += 1
            for _ in range(args.warmup):
                frame()
                with torch.cuda.stream(stream):
                    flush.add_(1.0)   # the first torch launch loads its module: keep it out of the timed region
            r.synchronize()
            torch.cuda.synchronize()
            start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                start.record(stream)
                for j in range(args.steps):
                    frame()
                    if j + 1 < args.steps:
                        flush.add_(1.0)
                stop.record(stream)
            r.synchronize()
            torch.cuda.synchronize()
            res[name] = {"ms_per_frame": start.elapsed_time(stop) / args.steps}
            print(f"[bench] {name}: {res[name]['ms_per_frame']:.2f} ms/frame", file=sys.stderr)
    finally:
        r.shutdown()
    t = res["temporal"]
    out = {"metric": "frames/s, 1920x1080 temporal accumulation, camera moving every frame (16 spp, depth 8)",
           "value": 1e3 / t["ms_per_frame"], "unit": "frames/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t["ms_per_frame"], "higher_is_better": True, "dtype": "f32",
           "data": "synthetic (seeded procedural scene)",
           "config": {"workload": "temporal_1080p_16spp_moving_camera", "width": W, "height": H, "spp": SPP,
                      "max_depth": DEPTH, "l2": "flushed between frames"}, "modes": res}
    print(json.dumps(out))


def run_profile_case(spec, tuning=()):
    """Two frames of the full-frame scene at a reduced size ("WxHxSPP"): the
    small case that ncu captures of single kernels run on.  tuning: kpt_tuning
    fields as "name=value" strings."""
    from kittlespt_gb300 import scenes as S
    from kittlespt_gb300.renderer import Renderer
    w, h, spp = (int(v) for v in spec.lower().split("x"))
    r = Renderer(0)
    r.initialize()
    sc = S.scene_full(w, h, spp, DEPTH)
    sc.sky_arith = 1   # as the full-frame workload
    r.load_scene(sc)
    if tuning:
        r.set_tuning(**{k: (float(v) if k == "grid_scale" else int(v)) for k, v in (t.split("=") for t in tuning)})
    for _ in range(2):
        r.execute_rendering(16.0, spp)
    r.synchronize()
    print(f"profile case {w}x{h}x{spp}: {r.stats().box_tests} box tests", file=sys.stderr)
    r.shutdown()


def run_batch_case(shared):
    """Two submissions of the 32-job batch (shared ray queues, or each job's
    frame a branch of the graph) and nothing else: the case that ncu launch
    lists of the batch run on."""
    from kittlespt_gb300.renderer import Batch, Renderer
    jobs = batch_jobs()
    rs = []
    for sc in jobs:
        r = Renderer(0)
        r.initialize()
        r.load_scene(sc)
        rs.append(r)
    with Batch(0) as b:
        b.shared = shared
        for _ in range(2):
            b.submit(rs, [sc.spp for sc in jobs])
            _, ms = b.wait()
    print(f"batch case ({'shared queues' if shared else 'branches'}): {ms:.2f} ms", file=sys.stderr)
    for r in rs:
        r.shutdown()


def run_adjoint_case(spec):
    """Two adjoint evaluations of the differentiation scene at a reduced size
    ("WxHxSPP") with a random adjoint image: the small case that ncu captures
    of the adjoint's kernels run on."""
    import torch
    from kittlespt_gb300 import _lib as K
    from kittlespt_gb300 import scenes as S
    from kittlespt_gb300.renderer import Renderer
    w, h, spp = (int(v) for v in spec.lower().split("x"))
    sc = adjoint_scene()
    sc.width, sc.height = w, h
    sc.camera = S.Camera.look_at((0.0, 1.0, 5.0), (0.0, 0.0, 0.0), 45.0, w, h)
    r = Renderer(0)
    r.initialize()
    r.load_scene(sc)
    adj = torch.rand((h, w, 4), device="cuda", generator=torch.Generator("cuda").manual_seed(1))
    n = C.c_int()
    K.check(r._L.kpt_adjoint_param_count(r.ctx, C.byref(n)))
    g = torch.zeros(n.value, dtype=torch.float64, device="cuda")
    for _ in range(2):
        K.check(r._L.kpt_adjoint_device(r.ctx, 0, spp, adj.data_ptr(), g.data_ptr(), None))
    r.synchronize()
    print(f"adjoint case {w}x{h}x{spp}: |grad| {float(g.norm()):.6g}", file=sys.stderr)
    r.shutdown()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the 32 mixed jobs, batched against one by one")
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip the differentiation workload's gradient evaluations/s")
    ap.add_argument("--no-megakernel", action="store_true",
                    help="skip timing the reference's own CUDA megakernel on the same scene")
    ap.add_argument("--workload", default="frame",
                    choices=["frame", "batch", "adjoint", "traversal", "blas", "upscale", "temporal"],
                    help="frame: the 1080p full-frame metric; batch: 32 mixed jobs, batched vs one by one; "
                         "adjoint: gradient evaluations/s of the path-replay adjoint; "
                         "traversal: rays/s on 2M random triangles; blas: BLAS build on upload, host vs device; "
                         "upscale: 1080p output rendered at 1/2.5 and upscaled, bilinear and FSR; "
                         "temporal: 1080p temporal accumulation with a moving camera")
    ap.add_argument("--profile-case", default=None, metavar="WxHxSPP",
                    help="render two frames of the full scene at this size and exit (small case for ncu)")
    ap.add_argument("--tuning", action="append", default=[], metavar="NAME=VALUE",
                    help="with --profile-case: a kpt_tuning field for its renderer (repeatable)")
    ap.add_argument("--adjoint-case", default=None, metavar="WxHxSPP",
                    help="run two adjoint evaluations of the differentiation scene at this size and exit "
                         "(small case for ncu)")
    ap.add_argument("--batch-case", default=None, choices=["shared", "branches"],
                    help="submit the 32-job batch twice in this mode and exit (case for ncu launch lists)")
    args = ap.parse_args()
    if args.batch_case:
        run_batch_case(args.batch_case == "shared")
        return
    if args.profile_case:
        run_profile_case(args.profile_case, args.tuning)
        return
    if args.adjoint_case:
        run_adjoint_case(args.adjoint_case)
        return
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    elif args.workload == "traversal":
        run_traversal(args)
    elif args.workload == "blas":
        run_blas(args)
    elif args.workload == "upscale":
        run_upscale(args)
    elif args.workload == "temporal":
        run_temporal(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
