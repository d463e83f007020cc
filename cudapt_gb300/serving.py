"""Batched render serving over the C ABI (gbpt_server_*) and the harness of
the benchmark's serving configuration.

``Server`` submits requests of any size from Python; the library's worker
threads run them concurrently on their own renderers and CUDA streams, admit
them by free HBM and choose the wavefront's scheduling knobs with an online
autotuner (include/gbpt.h, csrc/server.cpp).  ``poisson_workload`` draws the
serving configuration (scenes of the three benchmark configurations,
resolutions {128^2, 256^2, 512^2, 1024x768}, {4, 16, 64} samples per pixel,
depth caps {6, 8, 10}) and ``run_poisson`` submits it at Poisson arrival
times and reports per-request latency percentiles and the aggregate
Mpaths/s.  The reference has no serving path: it renders one scene per
process (src/cudaRTBDPTStream.cu:134-169, 816-951).
"""
import ctypes
import time

import numpy as np

from . import layouts
from ._native import Request, RequestStatus, check, load
from .layouts import as_params

RESOLUTIONS = ((128, 128), (256, 256), (512, 512), (1024, 768))
SPP = (4, 16, 64)
DEPTHS = (6, 8, 10)


class Server:
    """gbpt_server: `workers` concurrent requests, `hbm_reserve` bytes of HBM kept free."""

    FIFO, SHORTEST_FIRST = 0, 1

    def __init__(self, workers=4, hbm_reserve=1 << 30, policy=SHORTEST_FIRST, graphs=True):
        h = ctypes.c_void_p()
        check(load().gbpt_server_create(int(workers), int(hbm_reserve), ctypes.addressof(h)))
        self._h = h
        self._keep = {}  # id -> objects the library reads until the request ends
        check(load().gbpt_server_set_policy(self._h, int(policy)))
        check(load().gbpt_server_set_graphs(self._h, 1 if graphs else 0))

    def submit(self, scene, cam, width, height, frames, mode=layouts.MODE_BDPT_SC, params=None, out=None):
        """Queue one request; `out` (float32, width*height*3, optional) receives the image.
        Returns the request id."""
        from . import camera as make_camera
        if isinstance(cam, dict):
            cam = make_camera(cam["pos"], cam["dir"], cam["up"], cam["fov"])
        q = Request()
        q.scene = scene.handle.value
        q.camera[:] = [float(x) for x in np.asarray(cam, np.float32).reshape(-1)[:10]]
        q.width, q.height, q.frames, q.mode = int(width), int(height), int(frames), int(mode)
        p = as_params(params) if params is not None else None
        q.params = p.ctypes.data if p is not None else None
        if out is not None:
            if out.dtype != np.float32 or out.size < width * height * 3 or not out.flags.c_contiguous:
                raise ValueError("out must be a contiguous float32 array of width*height*3")
            q.out_rgb = out.ctypes.data
        rid = ctypes.c_uint64()
        check(load().gbpt_server_submit(self._h, ctypes.addressof(q), ctypes.addressof(rid)))
        self._keep[rid.value] = (scene, out)
        return rid.value

    def wait(self, rid, timeout_ms=600_000, release=True):
        """Status of request `rid` once finished (raises GbptError on timeout);
        release: let the server forget it afterwards."""
        st = RequestStatus()
        check(load().gbpt_server_wait(self._h, int(rid), int(timeout_ms), ctypes.addressof(st)))
        self._keep.pop(int(rid), None)
        if release:
            check(load().gbpt_server_release(self._h, int(rid)))
        return st.as_dict()

    def tuned(self, mode, depth, width, height):
        """(walk_refill, tail_from, samples) the autotuner holds for a request class."""
        r, t, n = ctypes.c_uint32(), ctypes.c_int32(), ctypes.c_uint32()
        check(load().gbpt_server_tuned(self._h, int(mode), int(depth), int(width), int(height),
                                       ctypes.addressof(r), ctypes.addressof(t), ctypes.addressof(n)))
        return r.value, t.value, n.value

    def tuned_knobs(self, mode, depth, width, height):
        """Every knob the autotuner holds for a request class: dict(walk_refill,
        tail_from, bands, walk_ctas, tail_below, samples)."""
        p = layouts.default_params()
        n = ctypes.c_uint32()
        check(load().gbpt_server_tuned_params(self._h, int(mode), int(depth), int(width), int(height),
                                              p.ctypes.data, ctypes.addressof(n)))
        return dict(walk_refill=int(p["walk_refill"]), tail_from=int(p["tail_from"]), bands=int(p["bands"]),
                    walk_ctas=int(p["walk_ctas"]), tail_below=float(p["tail_below"]), samples=n.value)

    def close(self):
        """Finishes queued and running requests, then frees the renderers."""
        if getattr(self, "_h", None) and self._h.value:
            load().gbpt_server_destroy(self._h)
            self._h = ctypes.c_void_p()
        self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def poisson_workload(n=64, rate=200.0, seed=0, scenes=("cornell", "interior", "hall")):
    """The serving configuration's request list: (arrival_s, scene name, width,
    height, spp, depth) for n requests at Poisson rate `rate` per second."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    t -= t[0]
    out = []
    for i in range(n):
        w, h = RESOLUTIONS[int(rng.integers(len(RESOLUTIONS)))]
        out.append((float(t[i]), scenes[int(rng.integers(len(scenes)))], w, h,
                    SPP[int(rng.integers(len(SPP)))], DEPTHS[int(rng.integers(len(DEPTHS)))]))
    return out


def run_poisson(gb, workload, scene_objs, cameras, workers=4, hbm_reserve=1 << 30, warm=True,
                policy=Server.SHORTEST_FIRST, graphs=True):
    """Submit `workload` (from poisson_workload) at its arrival times.  Scenes
    are built and resident beforehand; result buffers are page-locked before
    the clock starts.  Returns a summary dict and the per-request statuses."""
    from . import _host_floats
    bufs = [_host_floats(w * h * 3) for (_, _, w, h, _, _) in workload]
    srv = Server(workers, hbm_reserve, policy, graphs)
    try:
        if warm:  # first-use costs (kernel loading, scene upload) outside the timed run
            ids = [srv.submit(scene_objs[name], cameras[name], 64, 64, 1,
                              params=gb.default_params(eye_depth_max=4, light_depth_max=4)) for name in scene_objs]
            for i in ids:
                srv.wait(i)
        t0 = time.perf_counter()
        ids, submitted = [], []
        for (at, name, w, h, spp, depth), (arr, _) in zip(workload, bufs):
            now = time.perf_counter() - t0
            if at > now:
                time.sleep(at - now)
            p = gb.default_params(eye_depth_max=depth, light_depth_max=depth)
            submitted.append(time.perf_counter() - t0)
            ids.append(srv.submit(scene_objs[name], cameras[name], w, h, spp, params=p, out=arr))
        st = [srv.wait(i) for i in ids]
        wall = time.perf_counter() - t0
    finally:
        srv.close()
        for arr, addr in bufs:
            if addr is not None:
                load().gbpt_host_unregister(addr)
    lat = np.array([s["latency_ms"] for s in st])
    paths = int(sum(s["paths"] for s in st))
    summary = {
        "requests": len(st),
        "failed": int(sum(1 for s in st if s["status"] != 0)),
        "p50_ms": round(float(np.percentile(lat, 50)), 2),
        "p99_ms": round(float(np.percentile(lat, 99)), 2),
        "mean_queue_ms": round(float(np.mean([s["queued_ms"] for s in st])), 2),
        "paths": paths,
        "wall_s": round(wall, 3),
        "mpaths_per_s": round(paths / wall / 1e6, 3),
        "workers": workers,
        "policy": "shortest first (aging)" if policy == Server.SHORTEST_FIRST else "fifo",
        "graphs": bool(graphs),
        "overlap": overlap(submitted, st, wall),
    }
    return summary, st


def overlap(submitted, statuses, wall):
    """How far requests ran side by side: each request runs from submit +
    queued_ms to submit + latency_ms; the share of the wall time with 0, 1, 2,
    ... requests running, the mean number running while any runs, and the
    summed run time over the wall time."""
    ev = []
    for t, s in zip(submitted, statuses):
        ev.append((t + s["queued_ms"] / 1e3, 1))
        ev.append((t + s["latency_ms"] / 1e3, -1))
    ev.sort()
    share, busy, run_sum = {}, 0.0, 0.0
    k, last = 0, 0.0
    for t, d in ev:
        span = max(t - last, 0.0)
        share[k] = share.get(k, 0.0) + span
        if k:
            busy += span
            run_sum += span * k
        k += d
        last = t
    share[0] = share.get(0, 0.0) + max(wall - last, 0.0)
    return {"share_of_wall_running": {str(n): round(v / wall, 3) for n, v in sorted(share.items())},
            "mean_running_while_busy": round(run_sum / busy, 2) if busy else 0.0,
            "run_time_over_wall": round(sum(s["run_ms"] for s in statuses) / 1e3 / wall, 2)}
