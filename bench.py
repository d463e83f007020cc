"""Benchmark of the GB300 streaming BDPT (plain "BDPTSC" mode).

Workload: the 1024x768 interior scene (20x10x30 room, 180 icospheres,
57,614 triangles), eye and light depth caps 10, one progressive frame per
step (786,432 camera paths), Philox seed 1234.  Prints one JSON line.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the reference algorithm's CPU implementation (the
oracle restatement, multithreaded over the machine's host cores) on the same
workload: the reference's own code is Windows/MSVC + CUDA 7.5 texture
references and does not build here.
"""
import argparse
import ctypes
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

# name -> (scene generator, width, height, mode, depth caps, description)
WORKLOADS = {
    "interior": ("interior", 1024, 768, 0, 10,
                 "plain streaming BDPT, procedural interior 20x10x30 room + 180 icospheres (57,614 tris), "
                 "1024x768, depth 10"),
    "hall": ("hall", 1280, 720, 0, 5,
             "plain streaming BDPT, procedural hall 40x8x40 + 144 pillars + 1200 boxes (332,180 tris), "
             "1280x720, depth 5"),
    "hall_adaptive": ("hall", 1280, 720, 1, 5,
                      "adaptive BDPT + bilateral (radius 4), procedural hall (332,180 tris), 1280x720, depth 5, "
                      "steady-state budgeted frames"),
    "cornell": ("cornell", 256, 256, 0, 8,
                "plain streaming BDPT, Cornell box (36 tris), 256x256, depth 8"),
}
WL = WORKLOADS["interior"]
WORKLOAD = WL[5]


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


def scene_and_camera():
    from cudapt_gb300 import scenes
    return getattr(scenes, WL[0])()


def params_for(gb_or_layouts, **kw):
    extra = dict(filter_radius=4) if WL[3] == 1 else {}
    extra.update(kw)
    return gb_or_layouts.default_params(eye_depth_max=WL[4], light_depth_max=WL[4], **extra)


W, H = WL[1], WL[2]


def run_cpu_sample(threads, rows, frames=1, seed=1234, bands=4):
    """Oracle (CPU restatement of the reference estimator) on `rows` full-width
    rows of the same workload, split into `bands` bands spread evenly over the
    image so that the sample's cost per path matches the whole frame's;
    returns (paths, seconds, build_seconds)."""
    import oracle
    from cudapt_gb300 import layouts
    (v, t, m), cam = scene_and_camera()
    sc = oracle.Scene(v, t, m)
    p = params_for(layouts, seed=seed)
    bands = max(1, min(bands, rows))
    per = [rows // bands + (1 if b < rows % bands else 0) for b in range(bands)]
    dt = 0.0
    for b, rb in enumerate(per):
        y0 = (H - rb) * b // max(bands - 1, 1)
        r = oracle.Renderer(W, rb, 0, p, threads=threads)
        r.set_window(0, y0, W, H)
        t0 = time.perf_counter()
        r.render(sc, cam, frames)
        dt += time.perf_counter() - t0
    return W * rows * frames, dt, sc.build_seconds


def bench_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    # bounded sample per step: a quarter of the frame's rows in 4 bands
    rows = int(os.environ.get("GBPT_REF_ROWS", str(H // 4)))
    for _ in range(args.warmup if args.warmup < 1 else 1):
        run_cpu_sample(threads, 4)
    paths = secs = 0.0
    for _ in range(args.steps):
        p, dt, build_s = run_cpu_sample(threads, rows)
        paths += p
        secs += dt
    v = paths / secs / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "Mpaths/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * secs / args.steps, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "width": W, "height": H, "paths_per_step": W * rows,
                   "sample": f"{W}x{rows} rows per step in 4 bands spread over the frame"},
        "cpu_baseline": {"value": round(v, 4), "unit": "Mpaths/s", "cores": threads, "kind": "port",
                         "sample": f"{W}x{rows} rows (4 bands) x {args.steps} steps, oracle FP32 estimator + restated BVH build "
                                   f"({build_s:.2f} s build)"},
        "e2e": {"value": round(v, 4), "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def bench_gpu(args):
    rank, world, local = dist_env()
    import cudapt_gb300 as gb
    from cudapt_gb300 import build as gbuild
    gbuild.build()
    if world > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
    if not gb.device_available():
        raise SystemExit("bench: no usable CUDA device")
    (v, t, m), cam = scene_and_camera()
    scene = gb.RTScene(v, t, m).build_bvh()
    build_s = scene.build_seconds
    if args.traversal == "wide":
        scene.set_traversal("wide")
    params = params_for(gb)
    np_ = W * H
    r = gb.RTRenderer(W, H, WL[3], params)

    flush = FlushBuffer()
    # warm-up (the adaptive workload first runs its uniform frames, so that
    # every timed step is a budgeted + filtered frame)
    warm = max(args.warmup, 0) + (int(params["warmup_frames"]) if WL[3] == 1 else 0)
    for _ in range(warm):
        r.render_frames(scene, cam, 1, stats=True)
    # timed: one frame per step, L2 flushed (256 MB device memset) before each
    ms = []
    phases = {"ms_trace": 0.0, "ms_shade": 0.0, "ms_light": 0.0, "ms_filter": 0.0, "ms_adapt": 0.0,
              "ms_total": 0.0}
    rays = 0
    paths = 0
    launches = 0
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            flush()
            st = r.render_frames(scene, cam, 1, stats=True)
            ms.append(st["ms_total"])
            rays += st["rays"]
            paths += st["paths"]
            launches += st["launches"]
            for k in phases:
                phases[k] += st[k]
    total_ms = float(np.sum(ms))
    value = paths / (total_ms / 1e3) / 1e6

    # the same frames with the wide traversal (opt-in; same hits except surfaces closer together
    # than the reference's origin push), timed the same way on a second renderer
    wide = None
    if args.traversal == "reference" and not args.no_wide:
        scene.set_traversal("wide")
        rw = gb.RTRenderer(W, H, WL[3], params)
        for _ in range(warm):
            rw.render_frames(scene, cam, 1, stats=True)
        wms, wpaths = [], 0
        for _ in range(args.steps):
            flush()
            st = rw.render_frames(scene, cam, 1, stats=True)
            wms.append(st["ms_total"])
            wpaths += st["paths"]
        wv = wpaths / (float(np.sum(wms)) / 1e3) / 1e6
        wide = {"value": round(wv * world, 3), "ms_per_step": round(float(np.mean(wms)), 4),
                "tree": "binary tree collapsed to 4 children per node, nearest child first",
                "hits": "the reference's closest hit except where two surfaces lie within its 1e-4 origin push "
                        "of each other (tests/test_wide.py; 0.8% of random rays in the Cornell box, whose "
                        "blocks stand on the floor)"}
        rw.close()
        scene.set_traversal("reference")

    # e2e through the public call with a host result buffer (D2H of the image each step)
    out = np.zeros(np_ * 3, np.float32)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r.render(scene, cam, stats=False)
    e2e_s = time.perf_counter() - t0
    e2e = paths / e2e_s / 1e6

    # work counters for the roofline (separate, untimed frame)
    r.set_counting(True)
    cst = r.render_frames(scene, cam, 1, stats=True)
    r.set_counting(False)
    # bytes per visited node: 32 B bounds + 8 B child words (reference order); 112 B per
    # wide node (4 boxes + 4 child codes); 48 B per triangle test
    node_bytes = 112 if args.traversal == "wide" else 40
    trace_bytes = node_bytes * (cst["nodes"] + cst["shadow_nodes"]) + 48 * (cst["tris"] + cst["shadow_tris"])
    # the counting frame runs the counting variants of the walks (slower): its work
    # counts, over the timed frames' mean walk time
    trace_ms = phases["ms_trace"] / max(args.steps, 1)
    achieved = trace_bytes / (trace_ms / 1e3) / 1e9 if trace_ms > 0 else None
    peak, peak_kind = load_peaks()

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        rows = int(os.environ.get("GBPT_CPU_ROWS", str(H)))  # the whole frame
        p, dt, bs = run_cpu_sample(threads, rows)
        cpu = {"value": round(p / dt / 1e6, 4), "unit": "Mpaths/s", "cores": threads, "kind": "port",
               "sample": f"{W}x{rows} rows (4 bands spread over the frame) of one uniform frame, oracle FP32 estimator "
                         f"({bs:.2f} s restated BVH build)"}

    serving = None
    if rank == 0 and not args.no_serving:
        serving = serving_run(gb)

    D = int(params["eye_depth_max"])
    traffic = profiled_traffic(args.workload)
    line = {
        "metric": METRIC, "value": round(value * world, 3), "unit": "Mpaths/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (procedural scene, seeded)",
        "config": {"workload": WORKLOAD, "width": W, "height": H, "paths_per_step": np_,
                   "eye_depth_max": D, "light_depth_max": D, "tris": int(len(t)),
                   "l2": "flushed before every timed step (256 MB device memset)",
                   "bvh_build_s": round(build_s, 4), "rays_per_s": round(rays / (total_ms / 1e3), 1),
                   "traversal": args.traversal,
                   "phase_ms_per_step": {k: round(v_ / args.steps, 4) for k, v_ in phases.items()},
                   "parallelism": "replicas" if world > 1 else "single"},
        "e2e": {"value": round(e2e * world, 3), "unit": "Mpaths/s", "h2d_bytes_per_step": 40,
                "d2h_bytes_per_step": np_ * 12},
        "roofline": {"bound": "hbm", "kernel": "k_walk + k_tail (closest-hit + shadow BVH walks of one frame)",
                     "achieved": round(achieved, 1) if achieved else None, "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4) if achieved else None, "peak_kind": peak_kind,
                     "traffic": traffic,
                     "algorithmic_bytes_per_frame": int(trace_bytes),
                     # the tree and triangles are L2-resident: the L2 side of the same walks
                     "l2": l2_side(args.workload, trace_ms)},
        "filter_roofline": filter_roofline(phases, args.steps, np_, peak) if WL[3] == 1 else None,
        "wide_traversal": wide,
        "learned_sampler": learned_sampler_summary(),
        "serving": serving,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "gpu_launches": launches,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def serving_run(gb, n=64, rate=200.0, seed=0, workers=4):
    """The batched-serving configuration: n requests arriving as a Poisson
    process (rate per second), each a scene of the three plain benchmark
    scenes, a resolution of {128^2, 256^2, 512^2, 1024x768}, {4, 16, 64}
    spp and depth cap {6, 8, 10}; BVHs resident on the device, `workers`
    requests in flight (cudapt_gb300.serving)."""
    from cudapt_gb300 import scenes, serving
    objs, cams = {}, {}
    for name in ("cornell", "interior", "hall"):
        (v, t, m), cam = getattr(scenes, name)()
        objs[name] = gb.RTScene(v, t, m).build_bvh()
        cams[name] = cam
    wl = serving.poisson_workload(n, rate, seed)
    summary, st = serving.run_poisson(gb, wl, objs, cams, workers=workers)
    summary["config"] = (f"{n} requests, Poisson {rate:g}/s (seed {seed}), scenes cornell/interior/hall, "
                         "resolution in {128^2, 256^2, 512^2, 1024x768}, spp in {4, 16, 64}, depth in {6, 8, 10}, "
                         "plain BDPT, image copied to page-locked host memory per request")
    summary["unit"] = "Mpaths/s (all requests' camera paths / wall time from first arrival to last completion)"
    for s_ in objs.values():
        s_.close()
    return summary


def l2_side(workload, trace_ms):
    """L2 bytes of one frame's walks (32-byte sectors, profiles/walk_traffic_<workload>.txt)
    over this run's walk time, with the walk kernel's L2 throughput in percent of
    peak as ncu reports it (profiles/k_walk_k_tail_interior_1024x768.md)."""
    b = profiled_traffic(workload, "l2_bytes_per_frame")
    if b is None or not trace_ms:
        return None
    return {"bytes_per_frame": b, "achieved_GBs": round(b / (trace_ms / 1e3) / 1e9, 1),
            "throughput_pct_of_peak_ncu": [21.5, 16.8],
            "note": "L2 serves the walks' node and triangle fetches that miss L1 (74-75% L1 hit rate); "
                    "L2 throughput 17-22% of peak: latency-bound, not bandwidth-bound"}


def filter_roofline(phases, steps, np_, peak):
    """Bilateral filter of a budgeted frame against its compulsory traffic: the colour,
    position and normal planes read (12 B per pixel each) and 12 B per pixel written."""
    ms = phases["ms_filter"] / steps
    if ms <= 0:
        return None
    planes = 3
    compulsory = (planes * 12 + 12) * np_
    radius = 4
    gbs = compulsory / (ms / 1e3) / 1e9
    return {"kernel": "k_bilateral_tile", "bound": "hbm", "ms_per_frame": round(ms, 4),
            "compulsory_bytes": compulsory, "achieved": round(gbs, 1), "peak": peak, "unit": "GB/s",
            "frac": round(gbs / peak, 4),
            "taps_per_pixel": (2 * radius + 1) ** 2,
            "algorithmic_bytes_naive": (2 * radius + 1) ** 2 * planes * 12 * np_}


def learned_sampler_summary():
    """Equal-time RMSE of the learned allocator over the plain PLL allocator (held-out hall
    scenes), from the committed report of tests/experiments/learned_sampler.py."""
    p = os.path.join(ROOT, "profiles", "learned_sampler_hall_320x180.md")
    if not os.path.exists(p):
        return None
    out = {"report": "profiles/learned_sampler_hall_320x180.md", "scenes": "hall seeds 21-25, 320x180",
           "equal_time_s": [0.25, 0.5, 1.0]}
    with open(p) as f:
        for ln in f:
            parts = ln.split()
            if len(parts) == 2 and parts[0].startswith("learned_over_plain_rmse_"):
                out[parts[0]] = float(parts[1])
    return out


def profiled_traffic(workload, key="traffic_bytes_per_frame"):
    """A figure of the BVH-walk launches of one frame from the committed ncu
    summary of this workload (profiles/walk_traffic_<workload>.txt, line
    ``<key> <n>``): DRAM bytes (read + write) by default, ``l2_bytes_per_frame``
    for the L2's; None when no capture exists."""
    p = os.path.join(ROOT, "profiles", f"walk_traffic_{workload}.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for ln in f:
            parts = ln.split()
            if len(parts) == 2 and parts[0] == key:
                return int(parts[1])
    return None


class FlushBuffer:
    """Writes 256 MB of device memory (twice the 126 MB L2) before a step."""

    def __init__(self):
        import torch
        self.torch = torch
        self.buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    def __call__(self):
        self.buf.fill_(1.0)
        self.torch.cuda.synchronize()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbpt", choices=["gbpt", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="interior", choices=sorted(WORKLOADS))
    ap.add_argument("--no-wide", action="store_true", help="skip the extra wide-traversal timing")
    ap.add_argument("--no-serving", action="store_true", help="skip the batched-serving run")
    ap.add_argument("--traversal", default="reference", choices=["reference", "wide"],
                    help="BVH walk order: the reference's (bit-exact, default) or the collapsed 4-wide tree")
    args = ap.parse_args()
    global WL, WORKLOAD, W, H
    WL = WORKLOADS[args.workload]
    WORKLOAD, W, H = WL[5], WL[1], WL[2]
    if args.impl == "reference":
        bench_reference(args)
    else:
        bench_gpu(args)


if __name__ == "__main__":
    main()
