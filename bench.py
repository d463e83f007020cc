"""Benchmark of the GB300 streaming BDPT.  Prints one JSON line.

Headline workload (``--workload hall``, the default): plain streaming BDPT
("BDPTSC") on the procedural 332,180-triangle hall (40x8x40 room, 12x12
pillars, 1200 displaced boxes, 4 lights) at 1280x720, eye and light depth
caps 5 (the reference's compile-time caps), one progressive frame (921,600
camera paths) per step, Philox seed 1234.  The same run also measures, on
rank 0, the other benchmark configurations as secondary figures:

* ``interior``: 1024x768, 20x10x30 room + 180 subdivision-3 icospheres
  (230,414 triangles), constant environment 0.1, depth 10, 64 spp;
* ``hall_adaptive``: the hall with the PLL adaptive allocator, 8 uniform
  frames then 24 budgeted frames (32 spp mean), bilateral radius 4;
* ``cornell``: the 36-triangle Cornell box, 256x256, depth 8, 16 spp;
* batched serving (64 Poisson requests, saturated and below saturation).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the reference algorithm's CPU path on the machine's host
cores: the oracle (a line-by-line restatement of the reference estimator,
whose BVH builder and traversal equal the reference's own compiled code)
over the same whole frames.  The reference's CUDA renderer is not run: it
does not build with CUDA 13 without editing its sources, and its light pass
writes past the end of its light-vertex buffer.
"""
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

METRIC = "BDPT Mpaths/s"

# name -> scene generator and kwargs, image size, renderer mode, depth cap, extra params,
# frames that make one image, description
WORKLOADS = {
    "hall": dict(scene=("hall", {}), W=1280, H=720, mode=0, depth=5, params={}, image_frames=32,
                 desc="plain streaming BDPT, procedural hall 40x8x40 + 144 pillars + 1200 boxes (332,180 tris), "
                      "1280x720, depth 5"),
    "interior": dict(scene=("interior", {"level": 3}), W=1024, H=768, mode=0, depth=10,
                     params={"env": (0.1, 0.1, 0.1)}, image_frames=64,
                     desc="plain streaming BDPT, procedural interior 20x10x30 room + 180 subdivision-3 icospheres "
                          "(230,414 tris), constant environment 0.1, 1024x768, depth 10"),
    "hall_adaptive": dict(scene=("hall", {}), W=1280, H=720, mode=1, depth=5,
                          params={"filter_radius": 4, "warmup_frames": 8}, image_frames=32,
                          desc="adaptive BDPT + bilateral (radius 4), procedural hall (332,180 tris), 1280x720, "
                               "depth 5, 8 uniform + 24 budgeted frames"),
    "cornell": dict(scene=("cornell", {}), W=256, H=256, mode=0, depth=8, params={}, image_frames=16,
                    desc="plain streaming BDPT, Cornell box (36 tris), 256x256, depth 8, 16 spp"),
}

# static per-ray issue figures of the walk kernels, from single-kernel ncu captures
ISSUE_PROFILES = {"hall": "profiles/k_walk_k_tail_hall_640x360.md", "interior": "profiles/k_walk_k_tail_interior_512x384.md"}
SMS, SCHEDULERS = 152, 4


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)  # the first sample lands before the timed work starts
        except (OSError, FileNotFoundError):
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
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def scene_and_camera(wl):
    from cudapt_gb300 import scenes
    name, kw = wl["scene"]
    return getattr(scenes, name)(**kw)


def params_for(mod, wl, **kw):
    extra = dict(wl["params"])
    extra.update(kw)
    return mod.default_params(eye_depth_max=wl["depth"], light_depth_max=wl["depth"], **extra)


def run_cpu_frames(wl, threads, budget_s, max_frames, seed=1234, scene=None):
    """The oracle (CPU restatement of the reference estimator, its BVH builder
    and traversal equal to the reference's compiled code) on whole frames of
    the workload: frames until `budget_s` of render time or `max_frames`.
    Returns (paths, render seconds, frames, build seconds)."""
    import oracle
    from cudapt_gb300 import layouts
    (v, t, m), cam = scene_and_camera(wl)
    sc = scene if scene is not None else oracle.Scene(v, t, m)
    p = params_for(layouts, wl, seed=seed)
    r = oracle.Renderer(wl["W"], wl["H"], wl["mode"], p, threads=threads)
    paths, secs, frames = 0, 0.0, 0
    while frames < max_frames and (frames == 0 or secs < budget_s):
        t0 = time.perf_counter()
        r.render(sc, cam, 1)
        secs += time.perf_counter() - t0
        paths += r.stats()["paths"]
        frames += 1
    return paths, secs, frames, sc.build_seconds, sc


def bench_reference(args, wl):
    """The reference arm: the CPU path on the host cores, whole frames of the
    same workload, one frame per step."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    (v, t, m), _ = scene_and_camera(wl)
    sc = oracle.Scene(v, t, m)
    run_cpu_frames(wl, threads, 0.0, 1, scene=sc)  # warm-up: one frame (page-in, thread start)
    paths, secs, frames, build_s, _ = run_cpu_frames(wl, threads, 1e9, args.steps, scene=sc)
    v_ = paths / secs / 1e6
    sample = (f"{frames} whole {wl['W']}x{wl['H']} frames (one per step) of the same workload, oracle FP32 "
              f"estimator on {threads} host threads ({build_s:.2f} s BVH build, reported separately)")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v_, 4), "unit": "Mpaths/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * secs / max(frames, 1), 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (procedural scene, seeded)",
        "config": {"workload": wl["desc"], "width": wl["W"], "height": wl["H"], "paths_per_step": wl["W"] * wl["H"],
                   "sample": "whole frames, one per step", "bvh_build_s": round(build_s, 3)},
        "cpu_baseline": {"value": round(v_, 4), "unit": "Mpaths/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(v_, 4), "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


class RankSync:
    """Barriers and max-over-ranks of the replicas (one process per GPU under
    torchrun; gloo on the host, no data-path collective); no-ops for one rank."""

    def __init__(self, world):
        self.dist = None
        if world > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        import torch
        if torch.cuda.is_available():
            torch.cuda.synchronize()
        if self.dist:
            self.dist.barrier()

    def max(self, x):
        if not self.dist:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())


class FlushBuffer:
    """Writes 256 MB of device memory (twice the 126 MB L2) before a step."""

    def __init__(self):
        import torch
        self.torch = torch
        self.buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    def __call__(self):
        self.buf.fill_(1.0)
        self.torch.cuda.synchronize()


PHASES = ("ms_trace", "ms_shade", "ms_light", "ms_filter", "ms_adapt", "ms_total")


def timed_frames(r, scene, cam, steps, flush):
    """`steps` frames, one per step, L2 flushed before each; device times from
    the library's CUDA events on the renderer's stream."""
    ph = {k: 0.0 for k in PHASES}
    rays = paths = launches = 0
    for _ in range(steps):
        flush()
        st = r.render_frames(scene, cam, 1, stats=True)
        rays += st["rays"]
        paths += st["paths"]
        launches += st["launches"]
        for k in PHASES:
            ph[k] += st[k]
    return ph, rays, paths, launches


def walk_bytes(r, scene, cam, traversal="reference"):
    """Algorithmic bytes of one frame's BVH walks, counted by the kernels in an
    untimed frame: 40 B per node visit (32 B bounds + 8 B child words; 112 B
    per wide node) and 48 B per triangle test, closest-hit and any-hit walks."""
    r.set_counting(True)
    cst = r.render_frames(scene, cam, 1, stats=True)
    r.set_counting(False)
    node_bytes = 112 if traversal == "wide" else 40
    return (node_bytes * (cst["nodes"] + cst["shadow_nodes"]) + 48 * (cst["tris"] + cst["shadow_tris"]), cst)


def read_profile(path):
    """``key value`` lines of a committed profile summary (figures taken from an
    ncu capture whose command the file names)."""
    p = os.path.join(ROOT, path)
    out = {}
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for ln in f:
            parts = ln.strip().strip("`").split()
            if len(parts) == 2:
                try:
                    out[parts[0]] = float(parts[1])
                except ValueError:
                    pass
    return out


def issue_side(name, trace_ms, rays_per_frame, sm_mhz):
    """Issue-slot use of the walk kernels: warp instructions per ray from a
    single-kernel ncu capture (static, the file is named), times this run's
    rays, over 152 SMs x 4 schedulers x the sampled SM clock x this run's
    walk time; lanes active per instruction from the same capture."""
    src = ISSUE_PROFILES.get(name)
    prof = read_profile(src) if src else None
    if not prof or "warp_inst_per_ray" not in prof or not trace_ms or not sm_mhz:
        return None
    inst = prof["warp_inst_per_ray"] * rays_per_frame
    slots = SMS * SCHEDULERS * sm_mhz * 1e6 * trace_ms / 1e3
    return {"frac": round(inst / slots, 4), "lanes_active_per_inst": prof.get("lanes_active_per_inst"),
            "lane_frac": round(inst / slots * prof.get("lanes_active_per_inst", 0.0) / 32.0, 4),
            "warp_inst_per_ray": prof["warp_inst_per_ray"],
            "static_source": src + " (instructions per ray and lanes per instruction; the rest measured in this run)"}


def measure_workload(gb, name, steps, warmup, flush, peak, sm_mhz=None):
    """One benchmark configuration on its own renderer: `steps` timed frames
    (budgeted frames for the adaptive one, after its uniform frames), the
    whole image (all its frames) timed once, and the walks' work rate."""
    wl = WORKLOADS[name]
    (v, t, m), cam = scene_and_camera(wl)
    scene = gb.RTScene(v, t, m).build_bvh()
    params = params_for(gb, wl)
    r = gb.RTRenderer(wl["W"], wl["H"], wl["mode"], params)
    warm = warmup + (int(params["warmup_frames"]) if wl["mode"] == 1 else 0)
    for _ in range(warm):
        r.render_frames(scene, cam, 1, stats=True)
    ph, rays, paths, launches = timed_frames(r, scene, cam, steps, flush)
    tb, _ = walk_bytes(r, scene, cam)
    # the whole image: its frames from a reset, one call each (uniform + budgeted for the adaptive one),
    # device time and camera paths summed over the frames
    r.reset()
    flush()
    img_ms, img_paths = 0.0, 0
    for _ in range(wl["image_frames"]):
        st = r.render_frames(scene, cam, 1, stats=True)
        img_ms += st["ms_total"]
        img_paths += st["paths"]
    trace_ms = ph["ms_trace"] / steps
    out = {"workload": wl["desc"], "tris": int(len(t)), "width": wl["W"], "height": wl["H"],
           "value": round(paths / (ph["ms_total"] / 1e3) / 1e6, 3), "unit": "Mpaths/s",
           "ms_per_frame": round(ph["ms_total"] / steps, 4), "frames_timed": steps,
           "rays_per_s": round(rays / (ph["ms_total"] / 1e3), 1),
           "phase_ms_per_frame": {k: round(x / steps, 4) for k, x in ph.items()},
           "image": {"frames": wl["image_frames"], "ms": round(img_ms, 3), "paths": int(img_paths),
                     "mpaths_per_s": round(img_paths / (img_ms / 1e3) / 1e6, 3)},
           "walk_work_rate": {"bytes_per_frame": int(tb), "achieved_GBs": round(tb / (trace_ms / 1e3) / 1e9, 1),
                              "frac_of_hbm": round(tb / (trace_ms / 1e3) / 1e9 / peak, 4)} if trace_ms else None}
    if name == "hall_adaptive":
        out["filter"] = filter_roofline(ph, steps, wl["W"] * wl["H"], peak, int(params["filter_radius"]), sm_mhz)
    r.close()
    scene.close()
    return out


FILTER_PROFILE = "profiles/k_bilateral_tile_hall_adaptive_1280x720.md"


def filter_roofline(phases, steps, np_, peak, radius, sm_mhz):
    """Bilateral filter of a budgeted frame.  It is bound by instruction issue
    (the per-tap weights): warp instructions per pixel from a one-kernel ncu
    capture of the same pass (static, the file is named) x this frame's pixels
    over the issue slots of its measured time at the sampled SM clock.  Beside
    it, the HBM work rate of its compulsory traffic (the colour, position and
    normal planes read, 12 B per pixel each, and 12 B per pixel written)."""
    ms = phases["ms_filter"] / steps
    if ms <= 0:
        return None
    planes = 3
    compulsory = (planes * 12 + 12) * np_
    gbs = compulsory / (ms / 1e3) / 1e9
    prof = read_profile(FILTER_PROFILE) or {}
    issue = None
    if prof.get("warp_inst_per_pixel") and sm_mhz:
        slots = SMS * SCHEDULERS * sm_mhz * 1e6 * ms / 1e3
        issue = {"frac": round(prof["warp_inst_per_pixel"] * np_ / slots, 4),
                 "warp_inst_per_pixel": prof["warp_inst_per_pixel"],
                 "static_source": FILTER_PROFILE + " (instructions per pixel at radius 4; the rest measured in this run)"}
    return {"kernel": "k_bilateral_tile", "bound": "issue", "ms_per_frame": round(ms, 4), "issue": issue,
            "hbm_work_rate": {"compulsory_bytes": compulsory, "achieved": round(gbs, 1), "peak": peak,
                              "unit": "GB/s", "frac": round(gbs / peak, 4)},
            "taps_per_pixel": (2 * radius + 1) ** 2,
            "algorithmic_bytes_naive": (2 * radius + 1) ** 2 * planes * 12 * np_}


def bench_gpu(args, wl):
    rank, world, local = dist_env()
    import cudapt_gb300 as gb
    from cudapt_gb300 import build as gbuild
    gbuild.build()
    if world > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
    if not gb.device_available():
        raise SystemExit("bench: no usable CUDA device")
    sync = RankSync(world)
    W, H = wl["W"], wl["H"]
    (v, t, m), cam = scene_and_camera(wl)
    scene = gb.RTScene(v, t, m).build_bvh()
    build_s = scene.build_seconds
    if args.traversal == "wide":
        scene.set_traversal("wide")
    params = params_for(gb, wl)
    np_ = W * H
    r = gb.RTRenderer(W, H, wl["mode"], params)
    peak, peak_kind = load_peaks()

    flush = FlushBuffer()
    # warm-up (the adaptive workload first runs its uniform frames, so that
    # every timed step is a budgeted + filtered frame)
    warm = max(args.warmup, 0) + (int(params["warmup_frames"]) if wl["mode"] == 1 else 0)
    for _ in range(warm):
        r.render_frames(scene, cam, 1, stats=True)
    with ClockSampler(0) as clk:
        sync.barrier()
        phases, rays, paths, launches = timed_frames(r, scene, cam, args.steps, flush)
        sync.barrier()
    clocks = clk.summary()
    # replicas: every rank renders the same frames; the job's time is the slowest rank's
    total_ms = sync.max(phases["ms_total"])
    value = paths / (total_ms / 1e3) / 1e6

    # e2e through the public call with a host result buffer (D2H of the image each step)
    sync.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r.render(scene, cam, stats=False)
    e2e_s = sync.max(time.perf_counter() - t0)
    sync.barrier()
    e2e = paths / e2e_s / 1e6

    trace_bytes, cst = walk_bytes(r, scene, cam, args.traversal)
    trace_ms = phases["ms_trace"] / max(args.steps, 1)
    achieved = trace_bytes / (trace_ms / 1e3) / 1e9 if trace_ms > 0 else None
    rays_per_frame = rays / max(args.steps, 1)
    prof_src = ISSUE_PROFILES.get(args.workload)
    prof = (read_profile(prof_src) or {}) if prof_src else {}

    extras = {}
    if rank == 0 and not args.no_extras:
        # the same frames with the opt-in wide traversal, timed the same way on a second renderer
        if args.traversal == "reference":
            scene.set_traversal("wide")
            rw = gb.RTRenderer(W, H, wl["mode"], params)
            for _ in range(warm):
                rw.render_frames(scene, cam, 1, stats=True)
            wph, _, wpaths, _ = timed_frames(rw, scene, cam, args.steps, flush)
            extras["wide_traversal"] = {
                "value": round(wpaths / (wph["ms_total"] / 1e3) / 1e6, 3),
                "ms_per_step": round(wph["ms_total"] / args.steps, 4),
                "tree": "binary tree collapsed to 4 children per node, nearest child first (opt-in)",
                "hits": "the reference's closest hit except where two surfaces lie within its 1e-4 origin push of "
                        "each other (tests/test_wide.py)"}
            rw.close()
            scene.set_traversal("reference")
        others = {}
        for name in WORKLOADS:
            if name != args.workload:
                steps = 24 if name == "hall_adaptive" else max(4, min(args.steps, 10))
                others[name] = measure_workload(gb, name, steps, 2, flush, peak, clocks.get("sm_mhz"))
        extras["other_configs"] = others

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        p_, dt, frames, bs, _ = run_cpu_frames(wl, threads, 10.0, 40)
        cpu = {"value": round(p_ / dt / 1e6, 4), "unit": "Mpaths/s", "cores": threads, "kind": "port",
               "sample": f"{frames} whole {W}x{H} frames of the same workload (about 10 s), oracle FP32 estimator "
                         f"({bs:.2f} s BVH build, reported separately)"}

    if rank == 0 and not args.no_serving:
        extras["serving"] = serving_run(gb)

    line = {
        "metric": METRIC, "value": round(value * world, 3), "unit": "Mpaths/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (procedural scene, seeded)",
        "config": {"workload": wl["desc"], "width": W, "height": H, "paths_per_step": np_,
                   "eye_depth_max": wl["depth"], "light_depth_max": wl["depth"], "tris": int(len(t)),
                   "l2": "flushed before every timed step (256 MB device memset)",
                   "bvh_build_s": round(build_s, 4), "rays_per_s": round(rays / (total_ms / 1e3), 1),
                   "traversal": args.traversal,
                   "phase_ms_per_step": {k: round(v_ / args.steps, 4) for k, v_ in phases.items()},
                   "parallelism": "replicas" if world > 1 else "single"},
        "e2e": {"value": round(e2e * world, 3), "unit": "Mpaths/s", "h2d_bytes_per_step": 40,
                "d2h_bytes_per_step": np_ * 12},
        "roofline": {
            "bound": "hbm", "kernel": "k_walk + k_tail (closest-hit + shadow BVH walks of one frame)",
            "achieved": round(achieved, 1) if achieved else None, "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4) if achieved else None, "peak_kind": peak_kind,
            "note": "work rate: algorithmic walk bytes (40 B per node visit, 48 B per triangle test, counted by the "
                    "kernels in an untimed frame of this run) over this run's walk time; the tree is L2-resident, "
                    "so DRAM carries a small part of these bytes and the issue side below is the real limit",
            "algorithmic_bytes_per_frame": int(trace_bytes),
            "traffic": int(prof["dram_bytes_per_path"] * np_) if "dram_bytes_per_path" in prof else None,
            "traffic_source": (f"{prof_src} (static: DRAM bytes per camera path of one frame's walk and tail launches in an "
                               f"ncu capture of a smaller frame of the same scene, times this frame's paths)")
            if "dram_bytes_per_path" in prof else None,
            "l2_bytes_per_frame": int(prof["l2_bytes_per_path"] * np_) if "l2_bytes_per_path" in prof else None,
            "issue": issue_side(args.workload, trace_ms, rays_per_frame, clocks.get("sm_mhz")),
        },
        "cpu_baseline": cpu,
        "clocks": clocks,
        "gpu_launches": launches,
        "extra_keys": sorted(extras),
    }
    line.update(extras)
    if rank == 0:
        print(json.dumps(line), flush=True)
    r.close()


def serving_run(gb, n=64, rate=200.0, seed=0, workers=4):
    """The batched-serving configuration: n requests arriving as a Poisson
    process, each a scene of the three plain benchmark scenes, a resolution of
    {128^2, 256^2, 512^2, 1024x768}, {4, 16, 64} spp and depth cap {6, 8, 10};
    BVHs resident on the device, `workers` requests in flight
    (cudapt_gb300.serving).  Run at the configuration's rate (about 10x the
    GPU's capacity: latency is queueing) and again at 0.6x the capacity that
    run measured (latency is service time)."""
    from cudapt_gb300 import scenes, serving
    objs, cams = {}, {}
    for name in ("cornell", "interior", "hall"):
        (v, t, m), cam = getattr(scenes, name)()
        objs[name] = gb.RTScene(v, t, m).build_bvh()
        cams[name] = cam
    wl = serving.poisson_workload(n, rate, seed)
    summary, st = serving.run_poisson(gb, wl, objs, cams, workers=workers)
    summary["rate_per_s"] = rate
    cap = summary["requests"] / summary["wall_s"]
    low_rate = round(0.6 * cap, 2)
    low, _ = serving.run_poisson(gb, serving.poisson_workload(n, low_rate, seed), objs, cams, workers=workers)
    low["rate_per_s"] = low_rate
    # the saturated run again with one worker: the gain of running requests side by side
    one, _ = serving.run_poisson(gb, wl, objs, cams, workers=1)
    out = {"saturated": summary, "below_saturation": low,
           "saturated_one_worker": {k: one[k] for k in ("mpaths_per_s", "wall_s", "p50_ms", "p99_ms")},
           "capacity_requests_per_s": round(cap, 2),
           "config": (f"{n} requests, Poisson {rate:g}/s and 0.6x measured capacity (seed {seed}), scenes "
                      "cornell/interior/hall, resolution in {128^2, 256^2, 512^2, 1024x768}, spp in {4, 16, 64}, "
                      "depth in {6, 8, 10}, plain BDPT, image copied to page-locked host memory per request"),
           "unit": "Mpaths/s (all requests' camera paths / wall time from first arrival to last completion)"}
    for s_ in objs.values():
        s_.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbpt", choices=["gbpt", "reference"])
    ap.add_argument("--workload", default="hall", choices=sorted(WORKLOADS))
    ap.add_argument("--size", default=None, help="WxH override (profiling captures of a smaller frame)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-extras", action="store_true", help="skip the wide walk and the other configurations")
    ap.add_argument("--no-serving", action="store_true", help="skip the batched-serving runs")
    ap.add_argument("--traversal", default="reference", choices=["reference", "wide"],
                    help="BVH walk order: the reference's (bit-exact, default) or the collapsed 4-wide tree")
    args = ap.parse_args()
    wl = dict(WORKLOADS[args.workload])
    if args.size:
        w, h = (int(x) for x in args.size.lower().split("x"))
        wl.update(W=w, H=h, desc=wl["desc"] + f" (frame size {w}x{h})")
    if args.warmup < 3:
        print("bench: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        bench_reference(args, wl)
    else:
        bench_gpu(args, wl)


if __name__ == "__main__":
    main()
