"""RMSE-vs-time experiments of CudaPT, headless.

Restates the "RMSE Experiment" group of ``CUDAPTWindow`` (src/cudapt.cpp:
130-140 defaults, :198-222 knobs, :267-337 the per-tick logic, :840-858
SetConvergedResult, :898-949 the two toggles, :951-966 CalculateRMSE):

* a converged image is captured first (``capture_converged``);
* the scene is reset (progressive accumulation restarts at frame 0) and
  frames are rendered one after another while the elapsed render time
  accumulates;
* ``collect`` -- "Collect Massive Data": every ``interval_s`` seconds of
  elapsed time the RMSE against the converged image is appended as a
  ``seconds, frames, RMSE`` row; after ``n_points`` rows the CSV is written
  (the reference's defaults: 5 s, 30 points);
* ``until`` -- "Collect RMSE": stop at a time limit, a frame count, or the
  first frame whose RMSE is at or below a limit, and report that frame.

Elapsed time is the wall-clock time of the ``gbpt_render`` calls, which
include the device-to-host copy of the image, as the reference's ``Render``
did.  RMSE is computed on the GPU against the converged image
(``gbpt_renderer_rmse``) and is not part of the elapsed time (the reference
meant to subtract its RMSE time too, :300-301).
"""
import ctypes
import time

import numpy as np

from ._native import check, load, ptr


def renderer_rmse(renderer, converged):
    """RMSE of the renderer's current image against a converged W*H*3 image."""
    c = np.ascontiguousarray(converged, np.float32).reshape(-1)
    if c.size != renderer.width * renderer.height * 3:
        raise ValueError("converged image has the wrong size")
    out = ctypes.c_double()
    check(load().gbpt_renderer_rmse(renderer.handle, ptr(c), 0, ctypes.addressof(out)))
    return out.value


def capture_converged(renderer, scene, cam, frames):
    """Render `frames` progressive frames from scratch and return the image
    (CUDAPTWindow::SetConvergedResult of the current result)."""
    renderer.reset()
    for _ in range(max(frames - 1, 0)):
        renderer.render_frames(scene, cam, 1, stats=False)
    return renderer.render(scene, cam, stats=False).copy()


def collect(renderer, scene, cam, converged, interval_s=5.0, n_points=30, csv_path=None, max_frames=None):
    """"Collect Massive Data": rows (seconds, frames, RMSE) every interval_s of
    elapsed render time; writes them as CSV lines "s, n, rmse" when csv_path is given."""
    renderer.reset()
    rows = []
    elapsed, frames = 0.0, 0
    while len(rows) < n_points and (max_frames is None or frames < max_frames):
        t0 = time.perf_counter()
        renderer.render(scene, cam, stats=False)
        elapsed += time.perf_counter() - t0
        frames += 1
        if elapsed >= (len(rows) + 1) * interval_s:
            rows.append((elapsed, frames, renderer_rmse(renderer, converged)))
    if csv_path:
        with open(csv_path, "w") as f:
            for s, n, e in rows:
                f.write(f"{s:g}, {n}, {e:g}\n")
    return rows


def until(renderer, scene, cam, converged, seconds=0.0, frames=0, rmse_limit=0.0, max_frames=1 << 20):
    """"Collect RMSE": render until `seconds` of elapsed time, `frames` frames,
    or (rmse_limit > 0) the first frame whose RMSE <= rmse_limit.  Returns
    (seconds, frames, RMSE) of the frame that ended the run."""
    if not (seconds > 0 or frames > 0 or rmse_limit > 0):
        raise ValueError("give a time limit, a frame count or an RMSE limit")
    renderer.reset()
    elapsed, n, e = 0.0, 0, float("inf")
    while n < max_frames:
        t0 = time.perf_counter()
        renderer.render(scene, cam, stats=False)
        elapsed += time.perf_counter() - t0
        n += 1
        if rmse_limit > 0:
            e = renderer_rmse(renderer, converged)
            if e <= rmse_limit:
                break
        if (seconds > 0 and elapsed >= seconds) or (frames > 0 and n >= frames):
            break
    if rmse_limit <= 0:
        e = renderer_rmse(renderer, converged)
    return elapsed, n, e
