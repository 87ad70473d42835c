"""Benchmark: Mpaths/s of the wavefront path tracer on the 1000-sphere field
(default), or time to relMSE 0.01 of guided against plain rendering on the
occluded voxel hall (--workload voxel_hall).

Workload (the headline configuration): a seeded field of 1000 spheres on a
ground sphere (r = 1000 at y = -1000), centres uniform in [-11, 11] x [0.2, 1.2]
x [-11, 11], radii lognormal(mu = -1.6, sigma = 0.3), 60% lambertian (albedo
U[0,1]^3), 25% GGX metal (albedo U[0.5,1]^3, roughness U[0.02, 0.6]), 15%
dielectric (ior 1.5), lit by a 1024 x 512 equirectangular sky (gradient plus a
Gaussian sun lobe of angular radius 0.5 degrees and peak radiance 5e4)
importance-sampled by alias table; 1920 x 1080, 256 spp, max depth 16. All
inputs are synthetic and seeded; no dataset is involved.

One step = one full render of that frame (530.8 M paths). `value` times the
renders with the scene and the film resident in HBM (mypbr_gpu_render_device
on the current stream, CUDA events); `e2e` times the C-ABI call a user makes
with host buffers: mypbr_gpu_scene_create (uploads the flat scene) +
mypbr_gpu_render (renders, copies the FP64 frame back) + destroy.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--spp S]
  python bench.py --workload voxel_hall [--hall-width 1920] [--ref-spp 65536] [--repeats 4] [--repeat-spp 1024]
  python bench.py --workload cornell | triangle_room | batch
  python bench.py --workload hall_render [--hall-size 128] [--hall-width 256] [--spp 96] [--hidden 8]
                  [--per-wave 8]      (one render; the profiling case of the guiding kernels)

voxel_hall: the 512^3 voxel world lit through six slits (workloads.py),
rendered at --hall-width x 9/16 with max depth 16. relMSE = mean over pixels
and channels of (x - r)^2 / (r^2 + 0.01) against a plain render at --ref-spp
samples (FP64 film), minus the reference's own noise: the reference is the
mean of two independent half-spp renders, whose difference estimates that
noise (relMSE_raw in each point is the uncorrected value). The time to
target comes from --repeats independent renders of each method at
--repeat-spp (a fresh network for every guided one): their mean relMSE gives
c in relMSE = c/spp, and the time is c/0.01 samples at their mean seconds
per sample. With --curve each method also renders at doubling spp (a
fresh, untrained network for every guided render, so training time is
inside each timing) until relMSE <= 0.01 or --max-spp, reported as the
curve (with the time to
target that curve alone gives: interpolated log-log between the bracketing
renders, or extrapolated from the three highest-spp ones; single renders
are dominated by a few fireflies). The oracle is the plain estimator
itself, so the CPU figure is the plain method's spp to target at the
oracle's measured seconds per spp (a bounded run on every host core).

cornell / triangle_room: Mpaths/s of C1 / C3 (render_ex, scene resident),
the oracle beside it; with --hidden H the triangle room also renders guided
and compares plain and guided relMSE at equal time against --c3-ref-spp.
batch: C4, 64 scenes in one mypbr_gpu_render_batch call with feature guides,
every frame denoised, per-scene relMSE against 4x-spp renders.
--traversal 0..5 picks the walk (the scene's default: postponed leaves where
triangles fill most leaves, else binary; lanes taking new rays; 4-wide tree;
postponed leaves; plain binary; 8-wide tree with quantised boxes), --block
the threads per block.

--impl reference times the CPU implementation of the same path (the FP64
restatement of the reference's camera::render in oracle/, on every host core)
on a bounded sample of the same workload. With N > 1 (torchrun) every rank
renders its own independent set of samples of the frame (weak scaling, no
collective inside the timed region); rank 0 prints the JSON line.
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WIDTH, HEIGHT = 1920, 1080
# k_extend as ncu measured it (profiles/k_extend_sphere_field_1080p.md: the
# capture command, the figures and the commit they were taken at; re-taken
# whenever k_extend changes): DRAM bytes per ray of bounce 0 of a 4-spp frame
# (ray records in, hit records and queue entries out, the tree staying in L2)
# and the issue figures of bounces 0 and 1.
EXTEND_PROFILE = {
    "profile": "profiles/k_extend_sphere_field_1080p.md",
    "commit": "c7bbfab",
    "dram_bytes": 298.96e6 + 135.59e6, "rays": 8294400,
    "issue_active_frac": [0.600, 0.620], "threads_per_instruction": [26.57, 12.92],
}
EXTEND_DRAM_BYTES_PER_RAY = EXTEND_PROFILE["dram_bytes"] / EXTEND_PROFILE["rays"]
METRIC = "Mpaths/s at 1080p"
UNIT = "Mpaths/s"


# ------------------------------------------------------------ the workload

from mypbr_gb300.workloads import (batch_scenes, cornell_scene, sphere_field_scene,  # noqa: E402
                                   triangle_room_scene, voxel_hall_scene)


WORKLOAD = {"workload": "sphere_field_1000_hdri", "width": WIDTH, "height": HEIGHT, "spp": 256, "max_depth": 16,
            "spheres": 1001, "environment": "1024x512 RGB float, alias-table sampled", "seed": 2,
            "l2": "inputs (path state, queues, FP64 film) exceed L2; L2 also flushed between steps",
            "guided": False}


# ------------------------------------------------------------ helpers

def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.file.close()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def flat_bytes(scene):
    """Bytes of the flat scene arrays (what mypbr_gpu_scene_create copies)."""
    from mypbr_gb300 import flat
    v = flat.view(scene)
    total = 0
    for k, a in v.items():
        if isinstance(a, np.ndarray):
            total += a.nbytes
    env = v["environment"]
    total += env.width * env.height * 3 * 4
    return total


def oracle_render_timed(scene, spp, threads, rows=None, row_stride=1):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    cam = scene.camera
    cam.samples_per_pixel = spp
    O = orc.OracleScene(scene)
    t = time.perf_counter()
    _, _, ex = O.render(cam, threads=threads, rows=rows, row_stride=row_stride)
    return time.perf_counter() - t, ex


def cpu_stride(scene, threads, budget_s):
    """The row stride of the CPU sample: every k-th row of the 1080p frame at
    the full 256 spp, k chosen from a short probe (every 108th row) so that
    the sample takes about budget_s seconds. Rows spread over the whole frame
    see every part of the image in proportion, unlike a band."""
    t1, ex1 = oracle_render_timed(scene, 256, threads, rows=(HEIGHT // 216, 0), row_stride=HEIGHT // 10)
    rate = ex1["paths"] / t1
    rows = max(4, min(HEIGHT, int(budget_s * rate / (WIDTH * 256))))
    return max(1, HEIGHT // rows)


def cpu_sample(scene, threads, stride):
    """Times the oracle on every `stride`-th row of the frame at 256 spp.
    Returns (Mpaths/s, paths, seconds, description)."""
    t, ex = oracle_render_timed(scene, 256, threads, rows=(stride // 2, 0), row_stride=stride)
    n_rows = ex["paths"] // (WIDTH * 256)
    desc = (f"every {stride}th row of 1920x1080 ({n_rows} rows from row {stride // 2}) at 256 spp: "
            f"{ex['paths']} paths in {t:.2f} s")
    return ex["paths"] / t / 1e6, ex["paths"], t, desc


# ------------------------------------------------------------ arms

def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import mypbr_gb300 as mp
    threads = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as d:
        scene = mp.load_scene(sphere_field_scene(d, spp=256))
        stride = cpu_stride(scene, threads, args.reference_budget)
        rates, seconds, paths = [], [], 0
        desc = ""
        for k in range(args.warmup + args.steps):
            mpaths, n, t, desc = cpu_sample(scene, threads, stride)
            if k >= args.warmup:
                rates.append(mpaths)
                seconds.append(t)
                paths = n
    value = statistics.mean(rates)
    frame_ms = WIDTH * HEIGHT * 256 / (value * 1e6) * 1e3
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": statistics.mean(seconds) * 1e3,
            "ms_per_step_is": f"the timed sample (every {stride}th row of the frame, {paths} paths); a full "
                              f"1080p frame at this rate would take {frame_ms:.0f} ms",
            "ms_per_frame_extrapolated": frame_ms,
            "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp64", "data": "synthetic", "config": WORKLOAD, "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "per step: " + desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch

    import mypbr_gb300 as mp
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    with tempfile.TemporaryDirectory() as d:
        scene = mp.load_scene(sphere_field_scene(d, spp=args.spp))
    cam = scene.camera
    cam.samples_per_pixel = args.spp
    cam.seed = 1000 + rank  # independent samples per rank
    gpu = mp.GpuScene(scene)
    mp.set_launch(gpu, block=args.block, traversal=args.traversal, wave_paths=args.wave_paths)
    L = mp.lib()
    c, o = cam.structs()
    w, h = c.image_width, c.image_height
    rad = torch.zeros((h, w, 3), dtype=torch.float64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # larger than the 129 MB L2
    stream = torch.cuda.current_stream(dev)

    def step(stats, timing):
        o.timing = int(timing)
        mp.check(L.mypbr_gpu_render_device(gpu.handle, ctypes.byref(c), ctypes.byref(o),
                                           ctypes.c_void_p(rad.data_ptr()), None, None, None,
                                           ctypes.c_void_p(stream.cuda_stream), ctypes.byref(stats)))

    for _ in range(args.warmup):
        flush.fill_(1)
        step(mp.RenderStatsStruct(), False)
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    times, launches = [], 0
    totals = {"ext": 0, "sh": 0}
    for _ in range(args.steps):
        flush.fill_(1)
        st = mp.RenderStatsStruct()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step(st, False)  # the production path: each wave a replayed CUDA graph
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
        launches += st.kernel_launches
        totals["ext"] += st.extension_rays
        totals["sh"] += st.shadow_rays
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    # one more frame, after the timed region, with every kernel launched on its
    # own between CUDA events: the kernels' shares and k_extend's launch time
    flush.fill_(1)
    kst = mp.RenderStatsStruct()
    step(kst, True)
    torch.cuda.synchronize()
    kernel_ms = {k: getattr(kst, k) for k in ("ms_extend", "ms_shade", "ms_shadow", "ms_generate", "ms_other")}
    total_ms = sum(times)
    if world > 1:
        t = torch.tensor([total_ms], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    paths_per_step = w * h * args.spp
    value = world * paths_per_step * args.steps / (total_ms * 1e-3) / 1e6

    # e2e through the C ABI with host buffers: upload, render, copy back
    host = np.zeros((h, w, 3))
    e2e_times = []
    h2d = flat_bytes(scene)
    o.timing = 0
    for k in range(max(1, args.e2e_steps) + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g2 = mp.GpuScene(scene)
        mp.set_launch(g2, block=args.block, traversal=args.traversal, wave_paths=args.wave_paths)
        mp.check(L.mypbr_gpu_render(g2.handle, ctypes.byref(c), ctypes.byref(o), ctypes.c_void_p(host.ctypes.data),
                                    None, None, None, 0, mp.PASS_CALLBACK(), None))
        g2.close()
        dt = time.perf_counter() - t0
        if k > 0:  # the first one warms the host-side allocations
            e2e_times.append(dt)
    e2e = world * paths_per_step / statistics.mean(e2e_times) / 1e6

    # relMSE of the last timed frame (256 spp) against a 65,536-spp render of
    # every 8th row, made after the timed region as two independent halves
    # whose difference measures the reference's own noise (taken out)
    quality = None
    if rank == 0 and args.headline_ref_spp > 0:
        frame = rad.cpu().numpy()
        rows = list(range(4, h, 8))
        halves = []
        o.timing = 0
        saved = (o.samples_per_pixel, o.seed, o.first_row, o.row_count)
        t0 = time.perf_counter()
        for seed in (777001, 777002):
            half = torch.zeros((h, w, 3), dtype=torch.float64, device=dev)
            o.samples_per_pixel = args.headline_ref_spp // 2
            o.seed = seed
            for j in rows:
                o.first_row, o.row_count = j, 1
                mp.check(L.mypbr_gpu_render_device(gpu.handle, ctypes.byref(c), ctypes.byref(o),
                                                   ctypes.c_void_p(half.data_ptr()), None, None, None,
                                                   ctypes.c_void_p(stream.cuda_stream), None))
            torch.cuda.synchronize()
            halves.append(half.cpu().numpy()[rows])
        o.samples_per_pixel, o.seed, o.first_row, o.row_count = saved
        ref = 0.5 * (halves[0] + halves[1])
        raw = rel_mse(frame[rows], ref)
        noise = reference_noise(halves[0], halves[1])
        quality = {"relmse": raw - noise, "relmse_raw": raw, "reference_noise": noise, "epsilon": 0.01,
                   "reference": f"{args.headline_ref_spp} spp (two independent halves), FP64 film, rows 4, 12, ... "
                                f"({len(rows)} of {h}), {time.perf_counter() - t0:.1f} s after the timed region",
                   "of": f"the last timed frame ({args.spp} spp)"}

    if rank == 0:
        # roofline of the dominant kernel, extend: algorithmic bytes per ray =
        # ray record read (origin + tmin, direction + pdf: 32 B) + queue index
        # (4 B) + hit record written (16 B)
        ms_ext = kst.ms_extend / max(kst.launches_extend, 1)
        bytes_per_ray = 52
        ext_per_launch = kst.extension_rays / max(kst.launches_extend, 1)
        achieved = bytes_per_ray * ext_per_launch / (ms_ext * 1e-3) / 1e9 if ms_ext > 0 else 0.0
        peak = None
        try:
            with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
                peak = json.load(f)["hbm_gbs"]
            peak_src = "measured"
        except Exception:
            peak, peak_src = 6800.0, "fallback"
        frame_ms = sum(kernel_ms.values())
        shares = {k: v / frame_ms for k, v in kernel_ms.items()}
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
                "config": dict(WORKLOAD, spp=args.spp, parallelism=f"samples x{world}", traversal=args.traversal,
                               block=args.block or 256, wave_paths=args.wave_paths or "default"),
                "gpu_launches": int(launches),
                "rays": {"extension_per_path": totals["ext"] / (paths_per_step * args.steps),
                         "shadow_per_path": totals["sh"] / (paths_per_step * args.steps),
                         "mrays_per_s": world * (totals["ext"] + totals["sh"]) / (total_ms * 1e-3) / 1e6},
                "kernel_time_share": shares,
                "kernel_time_share_of": "one extra frame after the timed region, each kernel between CUDA events",
                "roofline": {"bound": "hbm", "kernel": "k_extend", "achieved": achieved, "peak": peak,
                             "unit": "GB/s", "frac": achieved / peak if peak else None,
                             "traffic": EXTEND_DRAM_BYTES_PER_RAY * ext_per_launch,
                             "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of k_extend on bounce "
                                               f"0 of a 4-spp frame ({EXTEND_PROFILE['dram_bytes'] / 1e6:.1f} MB for "
                                               f"{EXTEND_PROFILE['rays']} camera rays, {EXTEND_PROFILE['profile']}, captured at commit "
                                               f"{EXTEND_PROFILE['commit']}), "
                                               "scaled to the rays of an average launch",
                             "peak_source": peak_src, "bytes_per_ray": bytes_per_ray,
                             "avg_launch_ms": ms_ext, "rays_per_launch": ext_per_launch,
                             # the walk's real bound is instruction issue under divergence: the
                             # same ncu capture's issue-slot utilisation and lanes per instruction
                             "issue": {"issue_active_frac": EXTEND_PROFILE["issue_active_frac"],
                                       "threads_per_instruction": EXTEND_PROFILE["threads_per_instruction"],
                                       "source": "ncu smsp__issue_active and smsp__thread_inst_executed_per_"
                                                 "inst_executed of k_extend, bounces 0 and 1 of a 4-spp frame ("
                                                 + EXTEND_PROFILE["profile"] + ", captured at commit "
                                                 + EXTEND_PROFILE["commit"] + ")"}},
                "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                        "d2h_bytes_per_step": int(w * h * 3 * 8)},
                "clocks": clk}
        if quality:
            line["quality"] = quality
        if world == 1 and not args.no_cpu_baseline:
            threads = os.cpu_count() or 1
            mpaths, _, _, desc = cpu_sample(scene, threads, cpu_stride(scene, threads, args.cpu_budget))
            line["cpu_baseline"] = {"value": mpaths, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def rel_mse(x, ref, eps=0.01):
    return float(np.mean((x - ref) ** 2 / (ref ** 2 + eps)))


def reference_noise(half_a, half_b, eps=0.01):
    """The relMSE that the reference's own noise adds to every comparison
    against it. The reference is the mean of two independent renders of half
    its spp each; per pixel (a - b)^2 / 4 estimates the variance of that mean
    without bias, so E[relMSE(x, ref)] = relMSE(x, truth) + this value."""
    ref = 0.5 * (half_a + half_b)
    return float(np.mean((half_a - half_b) ** 2 / 4.0 / (ref ** 2 + eps)))


def time_to_target(points, target):
    """points: [(spp, seconds, relMSE)] at increasing spp. Seconds to reach target."""
    prev = None
    for spp, t, e in points:
        if e <= target:
            if prev is None or prev[2] <= e:
                return t, "measured"
            # log-log interpolation between the bracketing renders
            f = (math.log(prev[2]) - math.log(target)) / (math.log(prev[2]) - math.log(e))
            return math.exp(math.log(prev[1]) + f * (math.log(t) - math.log(prev[1]))), "interpolated"
        prev = (spp, t, e)
    spp_needed = spp_to_target(points, target)
    spp, t, _ = points[-1]
    return t / spp * spp_needed, "extrapolated (relMSE ~ c/spp, c fitted to the three highest-spp renders)"


def spp_to_target(points, target):
    """The spp at which relMSE ~ c / spp reaches target, c the geometric mean of
    relMSE x spp over the three highest-spp renders (one render's relMSE is
    dominated by a few fireflies; three damp that)."""
    last = points[-3:]
    c = math.exp(sum(math.log(e * s_) for s_, _, e in last) / len(last))
    return c / target


def run_voxel_hall(args):
    import mypbr_gb300 as mp
    width = args.hall_width or 1920
    height = width * 9 // 16
    target = 0.01
    with tempfile.TemporaryDirectory() as d:
        scene = mp.load_scene(voxel_hall_scene(d, size=512, width=width, height=height, spp=64))
    cam = scene.camera
    G = mp.GpuScene(scene)

    def render(gs, spp, guided, seed):
        cam.samples_per_pixel = spp
        cam.guided = guided
        cam.seed = seed
        cam.samples_per_wave = 0
        t0 = time.perf_counter()
        img, _, _ = mp.render_ex(cam, gs)
        return img, time.perf_counter() - t0

    render(G, 16, 0, 7)  # warm-up: path buffers
    # the reference as two independent halves: their difference measures the
    # reference's own noise, which is taken out of every relMSE below (a 65,536-
    # spp plain reference still carries relMSE ~0.04 on this scene, four times
    # the target, so an uncorrected curve levels off above the target)
    ref_a, t_a = render(G, args.ref_spp // 2, 0, 12345)
    ref_b, t_b = render(G, args.ref_spp // 2, 0, 54321)
    ref, t_ref = 0.5 * (ref_a + ref_b), t_a + t_b
    floor = reference_noise(ref_a, ref_b)
    del ref_a, ref_b

    def error(img):
        raw = rel_mse(img, ref)
        return max(raw - floor, 1e-12), raw
    Gg = mp.GpuScene(scene)
    render(Gg, 64, args.hidden, 7)  # warm-up: guiding buffers and network
    mp.guide_configure(Gg, alpha=args.guide_alpha, depths=args.guide_depths, alpha_deep=args.guide_alpha_deep)
    mp.guide_schedule(Gg, steps_early=args.steps_early, steps_late=args.steps_late, max_steps=args.max_steps,
                      use_after=args.use_after, weight_cap=args.weight_cap)
    curves = {}
    for name, guided in (("plain", 0), ("guided", args.hidden)):
        pts = []
        spp = 16
        while spp <= args.max_spp and args.curve:
            if guided:  # an untrained network every time: training is inside each timing
                mp.guide_reset(Gg)
            img, t = render(Gg if guided else G, spp, guided, 1 + spp)
            e, raw = error(img)
            pts.append((spp, t, e, raw))
            print(f"{name} spp {spp}: {t:.3f} s relMSE {e:.5f} (raw {raw:.5f})", file=sys.stderr, flush=True)
            if e <= target / 2:
                break
            spp *= 2
        tt, how = time_to_target([p_[:3] for p_ in pts], target) if pts else (None, "no curve rendered")
        # the estimate that decides: independent renders at one spp, whose mean
        # relMSE gives the error constant c = relMSE x spp (one render's relMSE
        # swings by 3x or more with the fireflies it happens to catch)
        reps = []
        for r_ in range(args.repeats):
            if guided:
                mp.guide_reset(Gg)
            img, t = render(Gg if guided else G, args.repeat_spp, guided, 1000 + r_)
            reps.append((t, error(img)[0]))
            print(f"{name} repeat {r_} at {args.repeat_spp} spp: {t:.3f} s relMSE {reps[-1][1]:.5f}",
                  file=sys.stderr, flush=True)
        rep_t = float(np.mean([t_ for t_, _ in reps]))
        rep_e = float(np.mean([e_ for _, e_ in reps]))
        c = rep_e * args.repeat_spp
        curves[name] = {"time_to_target_s": rep_t / args.repeat_spp * c / target,
                        "how": f"mean relMSE of {args.repeats} independent renders at {args.repeat_spp} spp, "
                               "relMSE ~ c/spp",
                        "error_constant": c, "spp_to_target": c / target,
                        "repeats": [{"seconds": t_, "relMSE": e_} for t_, e_ in reps],
                        "curve_time_to_target_s": tt, "curve_how": how,
                        "points": [{"spp": s_, "seconds": t_, "relMSE": e_, "relMSE_raw": r_}
                                   for s_, t_, e_, r_ in pts]}
    # CPU: the oracle on all host cores, a bounded run, extrapolated as relMSE ~ 1/spp
    import oracle as orc
    threads = os.cpu_count() or 1
    O = orc.OracleScene(scene)
    spp = 4
    while True:
        cam.samples_per_pixel = spp
        t0 = time.perf_counter()
        cpu_img, _, _ = O.render(cam, threads=threads)
        cpu_t = time.perf_counter() - t0
        cpu_spp = spp
        if cpu_t > args.cpu_budget / 3 or spp >= 256:
            break
        spp *= 2
    cpu_e, _ = error(cpu_img)
    # the oracle is the plain estimator itself (same sampling, renders within
    # 3 sigma of each other), so it needs the spp the plain GPU curve needs;
    # its time is that many samples at its measured seconds per sample
    cpu_tt = cpu_t / cpu_spp * curves["plain"]["spp_to_target"]
    cpu_tt_own = cpu_t * cpu_e / target
    line = {"metric": "time to relMSE 0.01 on the occluded voxel hall, guided GPU", "value": curves["guided"]["time_to_target_s"],
            "unit": "s", "n_gpus": 1, "higher_is_better": False, "dtype": "fp32", "data": "synthetic",
            "config": {"workload": "voxel_hall_512", "width": width, "height": height, "max_depth": 16,
                       "reference_spp": args.ref_spp, "reference_seconds": t_ref, "relmse_eps": 0.01,
                       "reference_noise_relmse": floor,
                       "relmse": "against the reference, minus the reference's own noise (two independent "
                                 "halves; relMSE_raw is uncorrected)",
                       "guide_hidden_layers": args.hidden, "guide_alpha": args.guide_alpha,
                       "guide_alpha_deep": args.guide_alpha_deep, "guide_depths": args.guide_depths,
                       "guide_schedule": {"steps_early": args.steps_early, "steps_late": args.steps_late,
                                          "weight_cap": args.weight_cap,
                                          "max_steps": args.max_steps, "use_after": args.use_after},
                       "sky": "atmosphere (procedural, Earth densities, lit by the sun's settings)",
                       "sun": "elevation 40 azimuth 160 intensity 1000 angle 0.54"},
            "plain": curves["plain"], "guided": curves["guided"],
            "guided_speedup_vs_plain": curves["plain"]["time_to_target_s"] / curves["guided"]["time_to_target_s"],
            "cpu_baseline": {"time_to_target_s": cpu_tt, "cores": threads, "kind": "port",
                             "sample": f"{cpu_spp} spp in {cpu_t:.1f} s (relMSE {cpu_e:.4f}); time = the plain "
                                       "curve's spp to target x the oracle's seconds per spp",
                             "time_to_target_own_sample_s": cpu_tt_own},
            "guided_speedup_vs_cpu": cpu_tt / curves["guided"]["time_to_target_s"]}
    print(json.dumps(line), flush=True)


def render_rate(mp, scene, spp, steps, warmup, guided=0, block=0, traversal=0, tune=None, wave_paths=0):
    """Device-resident Mpaths/s of a scene (CUDA events around the render on
    the scene handle's stream is what mypbr_gpu_render_ex times). With tune
    (a dict), the autotuner picks the launch settings first and tune gets its
    choice."""
    cam = scene.camera
    cam.samples_per_pixel = spp
    cam.guided = guided
    G = mp.GpuScene(scene)
    mp.set_launch(G, block=block, wave_paths=wave_paths, traversal=traversal)
    if tune is not None:
        r = mp.autotune(cam, G)
        tune.update({k: r[k] for k in ("block", "traversal", "wave_paths")})
    times = []
    st = None
    for k in range(warmup + steps):
        cam.seed = 100 + k
        t0 = time.perf_counter()
        img, _, st = mp.render_ex(cam, G)
        if k >= warmup:
            times.append(time.perf_counter() - t0)
    G.close()
    t = statistics.median(times)
    return st["paths"] / t / 1e6, t, st, img


def relmse_against_reference(mp, scene, img, spp, ref_spp, row_stride):
    """relMSE (epsilon 0.01) of img against a ref_spp render of every
    row_stride-th row (every row for 1), made as two independent halves whose
    difference removes the reference's own noise."""
    cam = scene.camera
    cam.guided = 0
    G = mp.GpuScene(scene)
    h = cam.height()
    rows = list(range(row_stride // 2, h, row_stride))
    halves = []
    t0 = time.perf_counter()
    for seed in (888001, 888002):
        cam.samples_per_pixel = ref_spp // 2
        cam.seed = seed
        if row_stride == 1:
            half, _, _ = mp.render_ex(cam, G)
        else:
            half = np.zeros((h, cam.image_width, 3))
            for j in rows:
                cam.first_row, cam.row_count = j, 1
                band, _, _ = mp.render_ex(cam, G)
                half[j] = band[j]
            cam.first_row, cam.row_count = 0, 0
        halves.append(half[rows])
    G.close()
    cam.samples_per_pixel = spp
    ref = 0.5 * (halves[0] + halves[1])
    raw = rel_mse(img[rows], ref)
    noise = reference_noise(halves[0], halves[1])
    return {"relmse": raw - noise, "relmse_raw": raw, "reference_noise": noise, "epsilon": 0.01,
            "reference": f"{ref_spp} spp (two independent halves), FP64 film, "
                         + ("every row" if row_stride == 1 else f"every {row_stride}th row ({len(rows)} of {h})")
                         + f", {time.perf_counter() - t0:.1f} s after the timed renders",
            "of": f"the last timed frame ({spp} spp)"}


def equal_time_relmse(mp, scene, spp, args):
    """C3's equal-time comparison: a plain render at spp, a guided one (the
    network trained inside its own time, from scratch) given the same time,
    both against a plain render at --c3-ref-spp; relMSE = mean over pixels
    and channels of (x - r)^2 / (r^2 + 0.01)."""
    cam = scene.camera

    def render(spp_, guided, seed):
        G = mp.GpuScene(scene)
        mp.set_launch(G, block=args.block, traversal=args.traversal)
        cam.samples_per_pixel = spp_
        cam.guided = guided
        cam.seed = seed
        t0 = time.perf_counter()
        img, _, st = mp.render_ex(cam, G)
        secs = time.perf_counter() - t0
        G.close()
        return img, secs, st

    ref, t_ref, _ = render(args.c3_ref_spp, 0, 991)

    def rel(img):
        return float(np.mean((img - ref) ** 2 / (ref * ref + 0.01)))

    plain, t_plain, _ = render(spp, 0, 7)
    # the guided rate at this spp, then the spp that fills the plain render's time
    _, t_probe, _ = render(spp, args.hidden, 8)
    spp_g = max(1, int(spp * t_plain / t_probe))
    guided, t_guided, _ = render(spp_g, args.hidden, 9)
    cam.guided = 0
    return {"seconds_plain": t_plain, "seconds_guided": t_guided, "reference_spp": args.c3_ref_spp,
            "reference_seconds": t_ref, "relmse_eps": 0.01,
            "plain": {"spp": spp, "relmse": rel(plain)}, "guided": {"spp": spp_g, "relmse": rel(guided)},
            "hidden_layers": args.hidden,
            "relmse_ratio_plain_over_guided": rel(plain) / max(rel(guided), 1e-30)}


def run_simple(args, workload):
    """C1 (Cornell box, 256^2, 64 spp, depth 50) or C3 (the 2M-triangle room,
    1080p, 64 spp, depth 12): Mpaths/s, timed around mypbr_gpu_render_ex
    (scene resident, FP64 frame copied back), and the CPU oracle beside it."""
    import mypbr_gb300 as mp
    with tempfile.TemporaryDirectory() as d:
        if workload == "cornell":
            scene = mp.load_scene(cornell_scene(d))
            spp, cfg = 64, {"workload": "cornell_box_c1", "width": 256, "height": 256, "spp": 64, "max_depth": 50}
        else:
            scene = mp.load_scene(triangle_room_scene(d))
            spp, cfg = 64, {"workload": "triangle_room_2m", "width": 1920, "height": 1080, "spp": 64,
                            "max_depth": 12, "triangles": 1985856, "materials": "32 principled", "lights": 16}
    tune = {} if args.autotune else None
    value, t, st, img = render_rate(mp, scene, spp, args.steps, args.warmup, block=args.block,
                                    traversal=args.traversal, tune=tune, wave_paths=args.wave_paths)
    if tune:
        cfg = dict(cfg, launch=dict(tune, chosen_by="mypbr_gpu_autotune"))
    line = {"metric": "Mpaths/s", "value": value, "unit": "Mpaths/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "dtype": "fp32",
            "data": "synthetic", "config": cfg,
            "rays": {"extension_per_path": st["extension_rays"] / st["paths"],
                     "shadow_per_path": st["shadow_rays"] / st["paths"],
                     "mrays_per_s": (st["extension_rays"] + st["shadow_rays"]) / t / 1e6}}
    if workload == "triangle_room" and args.hidden:
        gv, gt, _, _ = render_rate(mp, scene, spp, max(1, args.steps // 2), 1, guided=args.hidden,
                                   block=args.block, traversal=args.traversal)
        line["guided"] = {"value": gv, "ms_per_step": gt * 1e3, "hidden_layers": args.hidden,
                          "note": "untrained network at the first render; later renders train further"}
        line["equal_time"] = equal_time_relmse(mp, scene, spp, args)
    if args.headline_ref_spp > 0:
        line["quality"] = relmse_against_reference(mp, scene, img, spp, args.headline_ref_spp,
                                                   1 if workload == "cornell" else 16)
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        h = scene.camera.height()
        rows = max(1, min(h, int(h * 0.02))) if workload == "triangle_room" else h
        t_cpu, ex = oracle_render_timed(scene, spp, threads, rows=(h // 2 - rows // 2, rows))
        line["cpu_baseline"] = {"value": ex["paths"] / t_cpu / 1e6, "unit": "Mpaths/s", "cores": threads,
                                "kind": "port", "sample": f"{rows} rows at {spp} spp ({ex['paths']} paths, {t_cpu:.1f} s)"}
    print(json.dumps(line), flush=True)


def run_batch(args):
    """C4: 64 scenes of uneven size, resolution and spp (half of them with a
    haze medium) rendered by one mypbr_gpu_render_batch call with albedo,
    normal and variance guides, then each frame denoised (5 iterations) on the
    device; one step is both. Aggregate Mpaths/s over the batch. Per scene,
    relMSE (epsilon 0.01) of the noisy and of the denoised frame against a
    render of the same scene at 4x the spp with another seed."""
    import torch

    import mypbr_gb300 as mp
    d = tempfile.mkdtemp()
    items = batch_scenes(d, count=args.batch_count)
    scenes, cams, bufs = [], [], []
    for path, width, spp in items:
        sc = mp.load_scene(path)
        G = mp.GpuScene(sc)
        cam = sc.camera
        cam.samples_per_pixel = spp
        cam.collect_features = 1
        # --batch-wave-paths in flight per job (8M: 64 handles' path buffers stay near 80 GB)
        cam.samples_per_wave = max(1, args.batch_wave_paths // (cam.height() * cam.image_width))
        scenes.append((sc, G))
        cams.append(cam)
        h, w = cam.height(), cam.image_width
        z = lambda *shape: torch.zeros(shape, dtype=torch.float64, device="cuda")  # noqa: E731
        bufs.append({"rad": z(h, w, 3), "alb": z(h, w, 3), "nrm": z(h, w, 3), "var": z(h, w), "out": z(h, w, 3)})
    jobs = [(G, cam, b["rad"].data_ptr(), b["alb"].data_ptr(), b["nrm"].data_ptr(), b["var"].data_ptr())
            for (sc, G), cam, b in zip(scenes, cams, bufs)]

    def denoise_all():
        for cam, b in zip(cams, bufs):
            mp.denoise(b["rad"].data_ptr(), b["alb"].data_ptr(), b["nrm"].data_ptr(), b["var"].data_ptr(),
                       cam.image_width, cam.height(), b["out"].data_ptr(), on_device=True)

    paths = sum(c.height() * c.image_width * c.samples_per_pixel for c in cams)
    mp.render_batch(jobs)  # warm-up: buffers, graphs
    denoise_all()
    torch.cuda.synchronize()
    times, t_render = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        mp.render_batch(jobs)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        denoise_all()
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
        t_render.append(t1 - t0)
    t = statistics.median(times)
    # one by one, for the batch's gain (render only)
    per_job = []
    for job in jobs:
        t0 = time.perf_counter()
        mp.render_batch([job])
        torch.cuda.synchronize()
        per_job.append(time.perf_counter() - t0)
    t_serial = sum(per_job)
    # references: each scene at 4x the spp, another seed
    refs = []
    for (sc, G), cam in zip(scenes, cams):
        rc = mp.Camera(*cam.structs())
        rc.samples_per_pixel = cam.samples_per_pixel * 4
        rc.collect_features = 0
        rc.seed = cam.seed + 7919
        rb = torch.zeros((cam.height(), cam.image_width, 3), dtype=torch.float64, device="cuda")
        mp.render_batch([(G, rc, rb.data_ptr())])
        refs.append(rb)
    torch.cuda.synchronize()

    def rel_mse(x, r):
        return float((((x - r) ** 2) / (r * r + 0.01)).mean())

    noisy = [rel_mse(b["rad"], r) for b, r in zip(bufs, refs)]
    denoised = [rel_mse(b["out"], r) for b, r in zip(bufs, refs)]
    line = {"metric": "Mpaths/s over a batch of 64 scenes", "value": paths / t / 1e6, "unit": "Mpaths/s",
            "n_gpus": 1, "steps": args.steps, "higher_is_better": True, "dtype": "fp32", "data": "synthetic",
            "ms_per_step": t * 1e3,
            "config": {"workload": "batch_64", "scenes": len(items), "paths": int(paths),
                       "paths_in_flight_per_job": args.batch_wave_paths,
                       "triangles": "10k..1M log-uniform (a third of the scenes)",
                       "resolutions": "64^2..1024^2 log-uniform", "spp": "16..1024 log-uniform",
                       "media": "every other scene: fog 0.02, albedo 0.9, g 0.6",
                       "step": "render with albedo/normal/variance guides + 5-iteration denoise of every frame"},
            "render_ms": statistics.median(t_render) * 1e3,
            "one_by_one_render_ms": t_serial * 1e3, "batch_speedup": t_serial / statistics.median(t_render),
            "longest_job_alone_ms": max(per_job) * 1e3,
            "rel_mse": {"epsilon": 0.01, "reference": "same scene at 4x spp, another seed",
                        "noisy_median": statistics.median(noisy), "denoised_median": statistics.median(denoised),
                        "noisy": [round(x, 5) for x in noisy], "denoised": [round(x, 5) for x in denoised]}}
    print(json.dumps(line), flush=True)


def run_hall_render(args):
    """One render of the voxel hall (the case the profiles of the guiding
    kernels are taken on): --hall-size cells a side, --hall-width pixels
    wide (9:16), --spp samples, --hidden layers (0: plain), --per-wave passes
    per wave (0: automatic)."""
    import mypbr_gb300 as mp
    with tempfile.TemporaryDirectory() as d:
        w = args.hall_width or 256
        scene = mp.load_scene(voxel_hall_scene(d, size=args.hall_size, width=w, height=w * 9 // 16, spp=args.spp))
    G = mp.GpuScene(scene)
    mp.set_launch(G, block=args.block, traversal=args.traversal)
    mp.guide_configure(G, alpha=args.guide_alpha, depths=args.guide_depths, alpha_deep=args.guide_alpha_deep)
    mp.guide_schedule(G, steps_early=args.steps_early, steps_late=args.steps_late, max_steps=args.max_steps,
                      use_after=args.use_after, weight_cap=args.weight_cap)
    cam = scene.camera
    cam.samples_per_pixel = args.spp
    cam.guided = args.hidden
    cam.samples_per_wave = args.per_wave
    cam.seed = 1
    cam.timing = int(args.plain_launches)
    t0 = time.perf_counter()
    img, _, st = mp.render_ex(cam, G)
    t = time.perf_counter() - t0
    print(json.dumps({"metric": "Mpaths/s", "value": st["paths"] / t / 1e6, "unit": "Mpaths/s", "seconds": t,
                      "config": {"workload": f"voxel_hall_{args.hall_size}", "width": w, "height": w * 9 // 16,
                                 "spp": args.spp, "guided_hidden_layers": args.hidden,
                                 "samples_per_wave": args.per_wave},
                      "mean_radiance": float(img.mean()), "stats": st}), flush=True)


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--spp", type=int, default=256)
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--cpu-budget", type=float, default=12.0, help="seconds of CPU work for cpu_baseline")
    p.add_argument("--reference-budget", type=float, default=5.0, help="seconds per reference step")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--headline-ref-spp", type=int, default=65536,
                   help="spp of the reference the headline frame's relMSE is taken against (0: skip)")
    p.add_argument("--workload", choices=["sphere_field", "voxel_hall", "cornell", "triangle_room", "batch",
                                          "hall_render"], default="sphere_field")
    p.add_argument("--hall-size", type=int, default=512)
    p.add_argument("--per-wave", type=int, default=0)
    p.add_argument("--plain-launches", action="store_true",
                   help="hall_render: every kernel launched on its own with events (profilers cannot look inside "
                        "graphs with conditional nodes)")
    p.add_argument("--traversal", type=int, default=0, choices=[0, 1, 2, 3, 4, 5],
                   help="0: the scene's default; 1: extend lanes take new rays as theirs finish; 2: the 4-wide "
                        "tree; 3: postponed leaves; 4: the plain binary walk; 5: the 8-wide tree with quantised "
                        "boxes")
    p.add_argument("--block", type=int, default=0, choices=[0, 128, 256])
    p.add_argument("--autotune", action="store_true", help="cornell / triangle_room: autotuned launch settings")
    p.add_argument("--wave-paths", type=int, default=0,
                   help="sphere_field / cornell / triangle_room: paths per wave (0: the library's default)")
    p.add_argument("--batch-count", type=int, default=64)
    p.add_argument("--batch-wave-paths", type=int, default=8 << 20, help="batch: paths in flight per job")
    p.add_argument("--hall-width", type=int, default=0,
                   help="voxel_hall (default 1920, the configuration's width) / hall_render (default 256): pixels "
                        "wide, 16:9")
    p.add_argument("--curve", action="store_true",
                   help="voxel_hall: also render the doubling-spp curve (the repeated renders decide the time to "
                        "target)")
    p.add_argument("--ref-spp", type=int, default=65536)
    p.add_argument("--c3-ref-spp", type=int, default=1024, help="spp of the triangle room's reference render")
    p.add_argument("--max-spp", type=int, default=32768)
    p.add_argument("--repeat-spp", type=int, default=1024,
                   help="voxel_hall: spp of the repeated renders that estimate each method's error constant")
    p.add_argument("--repeats", type=int, default=4, help="voxel_hall: renders per method at --repeat-spp")
    p.add_argument("--hidden", type=int, default=8, help="hidden layers of the guiding network")
    p.add_argument("--guide-alpha", type=float, default=0.5, help="voxel_hall: probability of sampling the mixture")
    p.add_argument("--guide-depths", type=int, default=4, help="voxel_hall: bounces that sample the mixture")
    p.add_argument("--guide-alpha-deep", type=float, default=-1.0,
                   help="voxel_hall: probability of sampling the mixture after the first bounce (below 0: alpha)")
    p.add_argument("--use-after", type=int, default=128, help="voxel_hall: training steps before the mixture is used")
    p.add_argument("--steps-early", type=int, default=16, help="voxel_hall: Adam steps after each early wave")
    p.add_argument("--steps-late", type=int, default=4, help="voxel_hall: Adam steps after each later wave")
    p.add_argument("--max-steps", type=int, default=1500, help="voxel_hall: training steps in all")
    p.add_argument("--weight-cap", type=float, default=256.0,
                   help="voxel_hall: a training record's weight at most this x its batch's mean (0: no cap)")
    args = p.parse_args()
    if args.workload != "sphere_field":
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
    if args.workload == "voxel_hall":
        run_voxel_hall(args)
        return
    if args.workload in ("cornell", "triangle_room"):
        run_simple(args, args.workload)
        return
    if args.workload == "batch":
        run_batch(args)
        return
    if args.workload == "hall_render":
        run_hall_render(args)
        return
    if args.warmup < 3 and args.impl == "ours":
        print("note: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
