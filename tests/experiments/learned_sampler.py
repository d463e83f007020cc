"""Equal-time RMSE of the learned sample allocator against the plain PLL
allocator, scored against FP64 reference images of the CPU oracle.

Protocol of the benchmark's learned-sampler configuration: hall scenes of the
procedural generator, seeds 1-20 train and 21-25 held out.  Training samples
(24 tile features -> centred 0.5 log tile MSE) come from plain adaptive runs,
their targets from 1024-frame renders of the same scene; Adam at lr 1e-3 on
batches of 4096 tiles.  For each held-out scene and each of several Philox
keys, both allocators render frame after frame; the RMSE against the scene's
FP64 image (tests/experiments/make_truth.py, 8192 passes, its own Philox key)
is taken every few frames outside the timed render calls, giving RMSE as a
function of render wall time.  Reported: the RMSE ratio learned / plain at
equal times, and the time the learned allocator needs to reach the plain
one's RMSE at each time (the target is <= 0.6).  The plain allocator starts
its budgeted frames after the reference's 5 uniform frames; the learned one
after `--learned-warmup` (2 by default: the network needs only the features
of two frames, where the heuristic's filtered-minus-raw error is still blind).

    python tests/experiments/learned_sampler.py --truth DIR [--out report.json]
        [--res 320x180] [--keys 3] [--seconds 0.25,0.5,1,2] [--steps 2000]
        [--gpu-truth-frames N] [--check-truth]

At 1280x720 the FP64 images are out of reach of the host (the oracle renders
8192 passes of 320x180 in about 25 minutes on 7 cores; 1280x720 is 16 times
that per scene), so `--gpu-truth-frames N` renders any missing reference image
on the GPU instead: N plain-BDPT frames of the same estimator in FP32 with the
FP64 images' Philox key (777), cached in DIR as gputruth_<seed>_<W>x<H>_<N>.npy.
`--check-truth` (at a resolution with FP64 images) renders the GPU image too
and reports its RMSE against the FP64 one beside the errors being compared.

Needs a GPU.  Writes a JSON report and prints a markdown summary.
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

import cudapt_gb300 as gb  # noqa: E402
from cudapt_gb300 import layouts, learned  # noqa: E402


def seeds(s):
    if "-" in s:
        a, b = (int(x) for x in s.split("-"))
        return list(range(a, b + 1))
    return [int(x) for x in s.split(",")]


def training_set(train_seeds, W, H, boxes, target_frames, warmup, snapshots):
    Xs, Ys = [], []
    for s in train_seeds:
        (v, t, m), cam = learned.hall_scene(s, boxes)
        scene = gb.RTScene(v, t, m).build_bvh()
        ref = learned.converged(gb, scene, cam, W, H, target_frames, seed=999)
        r = gb.RTRenderer(W, H, layouts.MODE_BDPT_SC_ADAP_BILAT, learned.adaptive_params(warmup_frames=warmup))
        r.set_mlp(None, collect=True)
        for f in range(1, max(snapshots) + 1):
            img = r.render(scene, cam, stats=False)
            if f in snapshots:
                Xs.append(r.features())
                Ys.append(learned.tile_targets(img, ref, W, H))
        r.close()
        scene.close()
    return np.concatenate(Xs), np.concatenate(Ys)


def curve(scene, cam, W, H, truth, net, warmup, key, seconds, every=4):
    """(wall seconds, RMSE) points of one allocator rendering until `seconds`."""
    r = gb.RTRenderer(W, H, layouts.MODE_BDPT_SC_ADAP_BILAT,
                      learned.adaptive_params(warmup_frames=warmup, request_id=key))
    r.set_mlp(net, collect=False)
    r.render(scene, cam, stats=False)  # kernels loaded, buffers allocated (frame 0 is rendered again)
    r.reset()
    el, frames, pts = 0.0, 0, []
    while el < seconds:
        t0 = time.perf_counter()
        r.render_frames(scene, cam, 1, stats=False)
        el += time.perf_counter() - t0
        frames += 1
        if frames % every == 0:
            pts.append((el, r.rmse(truth), frames))
    r.close()
    return pts


def truth_image(args, s, W, H):
    """The scene's reference image: the FP64 one when present, else (with
    --gpu-truth-frames) a long GPU render with the same Philox key."""
    fp64 = os.path.join(args.truth, f"truth_{s}_{W}x{H}_{args.truth_frames}.npy")
    if os.path.exists(fp64):
        return np.load(fp64).astype(np.float32), "fp64"
    if not args.gpu_truth_frames:
        raise SystemExit(f"no reference image {fp64} (render it with make_truth.py, or pass --gpu-truth-frames)")
    return gpu_truth(args, s, W, H), "gpu"


def gpu_truth(args, s, W, H):
    path = os.path.join(args.truth, f"gputruth_{s}_{W}x{H}_{args.gpu_truth_frames}.npy")
    if os.path.exists(path):
        return np.load(path)
    (v, t, m), cam = learned.hall_scene(s, args.boxes)
    scene = gb.RTScene(v, t, m).build_bvh()
    img = learned.converged(gb, scene, cam, W, H, args.gpu_truth_frames, seed=777).astype(np.float32)
    scene.close()
    os.makedirs(args.truth, exist_ok=True)
    np.save(path, img)
    return img


def at(pts, t):
    """RMSE at wall time t (the last point at or before t)."""
    best = pts[0][1]
    for el, e, _ in pts:
        if el <= t:
            best = e
    return best


def time_to(pts, target):
    """Wall time at which the RMSE first falls to `target` (None: never)."""
    for el, e, _ in pts:
        if e <= target:
            return el
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--truth", required=True, help="directory of make_truth.py images")
    ap.add_argument("--truth-frames", type=int, default=8192)
    ap.add_argument("--out", default="learned_sampler.json")
    ap.add_argument("--res", default="320x180")
    ap.add_argument("--boxes", type=int, default=1200)
    ap.add_argument("--train-seeds", default="1-20")
    ap.add_argument("--test-seeds", default="21-25")
    ap.add_argument("--keys", type=int, default=3, help="Philox keys (request ids) per held-out scene")
    ap.add_argument("--seconds", default="0.25,0.5,1,2")
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--target-frames", type=int, default=1024)
    ap.add_argument("--learned-warmup", type=int, default=2)
    ap.add_argument("--gpu-truth-frames", type=int, default=0,
                    help="render missing reference images on the GPU with this many frames")
    ap.add_argument("--check-truth", action="store_true",
                    help="also render the GPU reference where an FP64 one exists and compare the two")
    args = ap.parse_args()
    W, H = (int(x) for x in args.res.split("x"))
    secs = [float(x) for x in args.seconds.split(",")]
    t0 = time.time()
    X, Y = training_set(seeds(args.train_seeds), W, H, args.boxes, args.target_frames, args.learned_warmup,
                        snapshots=(args.learned_warmup, args.learned_warmup + 1, 5, 8, 14))
    t_data = time.time() - t0
    t0 = time.time()
    net, losses = learned.train(X, Y, steps=args.steps, batch=4096, lr=1e-3)
    t_train = time.time() - t0
    # the heuristic alone as a tile-error predictor: a least-squares line on
    # its own tile feature (log of the tile's mean filtered-minus-raw error)
    A = np.stack([X[:, 22], np.ones(len(X))], 1)
    coef = np.linalg.lstsq(A, Y, rcond=None)[0]
    rows, pred_rows, truth_rows = [], [], []
    for s in seeds(args.test_seeds):
        truth, kind = truth_image(args, s, W, H)
        if args.check_truth and kind == "fp64" and args.gpu_truth_frames:
            g = gpu_truth(args, s, W, H)
            truth_rows.append(dict(seed=s, gpu_vs_fp64_rmse=float(np.sqrt(np.mean((g.astype(np.float64) - truth) ** 2))),
                                   fp64_mean=float(truth.mean())))
        (v, t, m), cam = learned.hall_scene(s, args.boxes)
        scene = gb.RTScene(v, t, m).build_bvh()
        r = gb.RTRenderer(W, H, layouts.MODE_BDPT_SC_ADAP_BILAT,
                          learned.adaptive_params(warmup_frames=args.learned_warmup))
        r.set_mlp(None, collect=True)
        for f in range(1, 9):
            img = r.render(scene, cam, stats=False)
            if f in (args.learned_warmup, 5, 8):
                Xt, Yt = r.features(), learned.tile_targets(img, truth, W, H)
                pn = net.forward(Xt)
                pn = pn - pn.mean()
                ph = np.stack([Xt[:, 22], np.ones(len(Xt))], 1) @ coef
                ph = ph - ph.mean()
                pred_rows.append(dict(seed=s, frame=f, network=float(np.mean((pn - Yt) ** 2)),
                                      heuristic=float(np.mean((ph - Yt) ** 2)), constant=float(np.mean(Yt ** 2))))
        r.close()
        for key in range(args.keys):
            plain = curve(scene, cam, W, H, truth, None, 5, key, max(secs))
            lrn = curve(scene, cam, W, H, truth, net, args.learned_warmup, key, max(secs))
            row = dict(seed=s, key=key, truth=kind)
            for sec in secs:
                ep, el = at(plain, sec), at(lrn, sec)
                tt = time_to(lrn, ep)
                row[str(sec)] = dict(plain=ep, learned=el, ratio=el / ep, time_to_plain=(tt / sec) if tt else None)
            rows.append(row)
            print(json.dumps(row), flush=True)
        scene.close()
    summ = {}
    for sec in secs:
        r = np.array([row[str(sec)]["ratio"] for row in rows])
        tt = [row[str(sec)]["time_to_plain"] for row in rows]
        ttv = np.array([x for x in tt if x is not None])
        summ[str(sec)] = dict(geo_mean_ratio=float(np.exp(np.mean(np.log(r)))), min_ratio=float(r.min()),
                              max_ratio=float(r.max()), learned_better=int(np.sum(r < 1.0)), runs=len(r),
                              median_time_to_plain=float(np.median(ttv)) if len(ttv) else None,
                              never_reached=int(sum(x is None for x in tt)))
    rep = dict(resolution=[W, H], boxes=args.boxes, train_seeds=args.train_seeds, test_seeds=args.test_seeds,
               keys=args.keys, samples=int(len(X)), steps=args.steps, target_frames=args.target_frames,
               truth_frames=args.truth_frames, learned_warmup=args.learned_warmup,
               loss_first=float(losses[:10].mean()), loss_last=float(losses[-10:].mean()), data_seconds=t_data,
               train_seconds=t_train, summary=summ, rows=rows, tile_prediction=pred_rows, truth_check=truth_rows,
               gpu_truth_frames=args.gpu_truth_frames,
               tile_prediction_mse=dict(network=float(np.mean([p["network"] for p in pred_rows])),
                                        heuristic=float(np.mean([p["heuristic"] for p in pred_rows])),
                                        constant=float(np.mean([p["constant"] for p in pred_rows]))))
    with open(args.out, "w") as f:
        json.dump(rep, f, indent=1)
    for tr in truth_rows:
        print(f"seed {tr['seed']}: GPU reference vs FP64 reference RMSE {tr['gpu_vs_fp64_rmse']:.5f}")
    tp = rep["tile_prediction_mse"]
    print(f"held-out tile log-error prediction MSE: network {tp['network']:.4f}, heuristic line "
          f"{tp['heuristic']:.4f}, constant {tp['constant']:.4f}")
    print("| seconds | geo-mean RMSE learned / plain | range | learned better | median time to plain's RMSE |")
    print("|---|---|---|---|---|")
    for sec in secs:
        x = summ[str(sec)]
        mt = f"{x['median_time_to_plain']:.2f}" if x["median_time_to_plain"] is not None else "n/a"
        print(f"| {sec} | {x['geo_mean_ratio']:.3f} | {x['min_ratio']:.2f}-{x['max_ratio']:.2f} | "
              f"{x['learned_better']}/{x['runs']} | {mt} ({x['never_reached']} never) |")


if __name__ == "__main__":
    main()
