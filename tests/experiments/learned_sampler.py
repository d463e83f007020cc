"""Equal-time RMSE of the learned sample allocator against the plain PLL
allocator, scored against the FP64 host-rendered image of the CPU oracle.

Protocol of the benchmark's learned-sampler configuration: hall scenes of
the procedural generator, seeds 1-20 train and 21-25 held out; training
samples (tile features -> centred 0.5 log tile MSE) from plain adaptive
runs; Adam at lr 1e-3 on batches of 4096 tiles; for each held-out scene,
both allocators render for the same wall time and their images are scored by
RMSE against the FP64 oracle image (and, for reference, against a long GPU
render).  Resolution is reduced (320 x 180 by default) so that the FP64
images finish on the host in seconds.

    python tests/experiments/learned_sampler.py [--out report.json] [--steps N]
        [--res 320x180] [--seconds 0.25,0.5,1.0] [--fp64-frames 256]

Writes a JSON report and prints a markdown table.  Needs a GPU.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
import cudapt_gb300 as gb  # noqa: E402
from cudapt_gb300 import learned  # noqa: E402


def rmse(a, b):
    return float(np.sqrt(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default="learned_sampler.json")
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--res", default="320x180")
    ap.add_argument("--boxes", type=int, default=1200)
    ap.add_argument("--seconds", default="0.25,0.5,1.0")
    ap.add_argument("--fp64-frames", type=int, default=256)
    ap.add_argument("--train-seeds", default="1-20")
    ap.add_argument("--test-seeds", default="21-25")
    ap.add_argument("--weights", default=None, help="write the trained parameters here (.npy)")
    args = ap.parse_args()
    W, H = (int(x) for x in args.res.split("x"))
    rng = lambda s: list(range(int(s.split("-")[0]), int(s.split("-")[1]) + 1)) if "-" in s else [int(s)]
    train_seeds, test_seeds = rng(args.train_seeds), rng(args.test_seeds)
    secs = [float(x) for x in args.seconds.split(",")]
    t0 = time.time()
    Xs, Ys = [], []
    for s in train_seeds:
        X, Y = learned.samples_for_scene(gb, s, W, H, boxes=args.boxes)
        Xs.append(X)
        Ys.append(Y)
    X, Y = np.concatenate(Xs), np.concatenate(Ys)
    t_data = time.time() - t0
    t0 = time.time()
    net, losses = learned.train(X, Y, steps=args.steps, batch=4096, lr=1e-3)
    t_train = time.time() - t0
    if args.weights:
        np.save(args.weights, net.params)
    rows = []
    for s in test_seeds:
        (v, t, m), cam = learned.hall_scene(s, args.boxes)
        p = learned.adaptive_params()
        t1 = time.time()
        ref64 = oracle.render_fp64(oracle.Scene(v, t, m), p, W, H, cam, args.fp64_frames)
        t_fp64 = time.time() - t1
        scene = gb.RTScene(v, t, m).build_bvh()
        ref32 = learned.converged(gb, scene, cam, W, H, 4096)
        Xt, Yt = learned.samples_for_scene(gb, s, W, H, snapshots=(5, 10), boxes=args.boxes)
        pred = net.forward(Xt)
        pred -= pred.mean()
        row = dict(seed=s, fp64_seconds=t_fp64, fp64_vs_gpu4096=rmse(ref64, ref32),
                   tile_mse_model=float(np.mean((pred - Yt) ** 2)), tile_mse_const=float(np.mean(Yt ** 2)))
        for sec in secs:
            out = learned.equal_time(gb, s, net, sec, W, H, ref=ref32, boxes=args.boxes)
            for name in ("plain", "learned"):
                e32, frames, img = out[name]
                row[f"{name}_{sec}s"] = dict(frames=frames, rmse_fp64=rmse(img, ref64), rmse_gpu4096=e32)
        rows.append(row)
        print(json.dumps(row), flush=True)
    rep = dict(resolution=[W, H], boxes=args.boxes, train_seeds=train_seeds, test_seeds=test_seeds,
               samples=int(len(X)), steps=args.steps, loss_first=float(losses[:10].mean()),
               loss_last=float(losses[-10:].mean()), data_seconds=t_data, train_seconds=t_train, rows=rows)
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    with open(args.out, "w") as f:
        json.dump(rep, f, indent=1)
    print("| seed | seconds | plain frames | learned frames | plain RMSE (FP64) | learned RMSE (FP64) | ratio |")
    print("|---|---|---|---|---|---|---|")
    for row in rows:
        for sec in secs:
            a, b = row[f"plain_{sec}s"], row[f"learned_{sec}s"]
            print(f"| {row['seed']} | {sec} | {a['frames']} | {b['frames']} | {a['rmse_fp64']:.5f} | "
                  f"{b['rmse_fp64']:.5f} | {b['rmse_fp64'] / a['rmse_fp64']:.3f} |")


if __name__ == "__main__":
    main()
