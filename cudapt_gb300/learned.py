"""Training and evaluation of the learned sample allocator.

The network (cudapt_gb300.mlp, kernels in csrc/mlp.cu) maps the 24 features
of an 8x8 tile (``gbpt_renderer_features``) to pred = 1/2 log of the tile's
current mean squared error (up to a per-image constant); the PLL adaptive
mode then gives each tile a share of the frame's samples proportional to
exp(2 pred) / n_t (n_t: the tile's mean samples per pixel), spread inside the
tile by the plain heuristic (``gbpt_renderer_set_mlp``).

Why.  With n_t samples per pixel and per-pixel variances summing to V_t over
the tile, the tile's squared error is V_t / n_t; one more sample per pixel
lowers it by about V_t / n_t^2 = MSE_t / n_t, and spending each frame where
that gain is largest drives the allocation towards the fixed-budget optimum
n_t proportional to sqrt(V_t) while accounting for samples already spent.
The squared error of the current image against a converged one estimates
MSE_t, so the training target is 0.5 log(tile MSE), centred per image.

Protocol (the benchmark's learned-sampler configuration): hall scenes of the
procedural generator, seeds 1-20 for training and 21-25 held out; features
after the uniform warm-up and after budgeted frames of the plain allocator;
converged images from long plain renders; Adam at lr 1e-3 on batches of 4096
tiles; comparison at equal wall time by RMSE against a converged reference.
"""
import time

import numpy as np

from . import layouts, scenes
from .mlp import MLP

EPS = 1e-12


def tile_targets(img, ref, width, height):
    """0.5 * log(mean squared error of each 8x8 tile), centred; row-major tiles."""
    tx, ty = (width + 7) // 8, (height + 7) // 8
    d = (np.asarray(img, np.float64) - np.asarray(ref, np.float64)).reshape(height, width, 3)
    e = (d * d).mean(axis=2)
    pad = np.zeros((ty * 8, tx * 8))
    cnt = np.zeros((ty * 8, tx * 8))
    pad[:height, :width] = e
    cnt[:height, :width] = 1
    se = pad.reshape(ty, 8, tx, 8).sum(axis=(1, 3))
    n = cnt.reshape(ty, 8, tx, 8).sum(axis=(1, 3))
    t = 0.5 * np.log(se / n + EPS)
    return (t - t.mean()).reshape(-1).astype(np.float32)


def hall_scene(seed, boxes=300):
    return scenes.hall(seed=seed, boxes=boxes)


def adaptive_params(depth=5, **kw):
    base = dict(eye_depth_max=depth, light_depth_max=depth, warmup_frames=5, filter_radius=4)
    base.update(kw)
    return layouts.default_params(**base)


def converged(gb, scene, cam, width, height, frames, depth=5, seed=1234):
    """A long plain-BDPT render of the same estimator (the reference image);
    `seed`: its Philox key (another key than the renders it scores shares no
    samples with them)."""
    r = gb.RTRenderer(width, height, layouts.MODE_BDPT_SC, adaptive_params(depth, seed=seed))
    for _ in range(frames - 1):
        r.render_frames(scene, cam, 1, stats=False)
    img = r.render(scene, cam, stats=False).copy()
    r.close()
    return img


def samples_for_scene(gb, seed, width=320, height=180, snapshots=(5, 7, 10, 14), conv_frames=512, boxes=300,
                      warmup=5):
    """(features, targets) of one training scene at several points of a plain
    adaptive run (budgeted frames after `warmup` uniform ones); the targets'
    converged image has its own Philox key (999), so it shares no samples
    with the run it scores."""
    (v, t, m), cam = hall_scene(seed, boxes)
    scene = gb.RTScene(v, t, m).build_bvh()
    ref = converged(gb, scene, cam, width, height, conv_frames, seed=999)
    r = gb.RTRenderer(width, height, layouts.MODE_BDPT_SC_ADAP_BILAT, adaptive_params(warmup_frames=warmup))
    r.set_mlp(None, collect=True)
    X, Y = [], []
    for f in range(1, max(snapshots) + 1):
        img = r.render(scene, cam, stats=False)
        if f in snapshots:
            X.append(r.features())
            Y.append(tile_targets(img, ref, width, height))
    r.close()
    return np.concatenate(X), np.concatenate(Y)


def train(X, Y, steps=2000, batch=4096, lr=1e-3, seed=0, log_every=0):
    """Adam on mean squared error over random batches; returns (net, losses)."""
    net = MLP(seed=seed)
    rng = np.random.Generator(np.random.PCG64(seed))
    losses = []
    for s in range(steps):
        idx = rng.integers(0, len(X), batch)
        losses.append(net.train_step(X[idx], Y[idx], lr))
        if log_every and s % log_every == 0:
            print(f"step {s} loss {losses[-1]:.4f}", flush=True)
    return net, np.array(losses)


def equal_time(gb, seed, net, seconds, width=320, height=180, ref=None, conv_frames=1024, boxes=300):
    """RMSE against the reference after `seconds` of rendering, plain vs learned allocation.
    Returns dict(plain=(rmse, frames, image), learned=(rmse, frames, image))."""
    (v, t, m), cam = hall_scene(seed, boxes)
    scene = gb.RTScene(v, t, m).build_bvh()
    if ref is None:
        ref = converged(gb, scene, cam, width, height, conv_frames)
    out = {}
    for name, mlp in (("plain", None), ("learned", net)):
        r = gb.RTRenderer(width, height, layouts.MODE_BDPT_SC_ADAP_BILAT, adaptive_params())
        r.set_mlp(mlp, collect=False)
        r.render(scene, cam, stats=False)  # warm the kernels (frame 0 is re-rendered below)
        r.reset()
        elapsed, frames = 0.0, 0
        while elapsed < seconds:
            t0 = time.perf_counter()
            r.render(scene, cam, stats=False)
            elapsed += time.perf_counter() - t0
            frames += 1
        out[name] = (r.rmse(ref), frames, r.GetResult().copy())
        r.close()
    return out
