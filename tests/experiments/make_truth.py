"""FP64 reference images for the learned-sampler comparison, rendered on the
host by the CPU oracle (no GPU needed).

    python tests/experiments/make_truth.py --out DIR [--seeds 21-25] [--res 320x180]
        [--frames 8192] [--threads N]

For each held-out hall scene (the adaptive benchmark's generator at the given
seed, 1200 boxes) it renders `frames` progressive passes (one camera sample
per pixel each) of the reference estimator in double precision and writes
DIR/truth_<seed>_<W>x<H>_<frames>.npy (float64, W*H*3, row 0 at the bottom).
At 8192 passes the image's own Monte Carlo error is far below the errors the
comparison scores.  Its Philox key (--seed, 777) differs from the renders it
scores (1234), so it shares no samples with them.
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from cudapt_gb300 import learned  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--seeds", default="21-25")
    ap.add_argument("--res", default="320x180")
    ap.add_argument("--frames", type=int, default=8192)
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--boxes", type=int, default=1200)
    ap.add_argument("--seed", type=int, default=777, help="Philox key of the reference renders")
    args = ap.parse_args()
    W, H = (int(x) for x in args.res.split("x"))
    a, b = (int(x) for x in args.seeds.split("-")) if "-" in args.seeds else (int(args.seeds),) * 2
    os.makedirs(args.out, exist_ok=True)
    oracle.build()
    for seed in range(a, b + 1):
        path = os.path.join(args.out, f"truth_{seed}_{W}x{H}_{args.frames}.npy")
        if os.path.exists(path):
            continue
        (v, t, m), cam = learned.hall_scene(seed, args.boxes)
        t0 = time.time()
        params = learned.adaptive_params(seed=args.seed)
        img = oracle.render_fp64(oracle.Scene(v, t, m), params, W, H, cam, args.frames, threads=args.threads)
        np.save(path, img)
        print(f"seed {seed}: {time.time() - t0:.0f} s -> {path}", flush=True)


if __name__ == "__main__":
    main()
