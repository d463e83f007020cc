"""Row-band sharding of one image across ranks (world_size 2, gloo, CPU).

Pixels are independent and every path's random numbers are fixed by its
global pixel id, so each rank renders a band of rows and the gathered bands
equal the single-process image bit for bit; the light-vertex cache is
replicated (same key and frame on every rank) and the one global scalar of
the adaptive mode (the error sum) is an all-reduce.  Runs the oracle: the
pool's boxes carry one GPU, so the sharded path is exercised on host ranks.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
dist = pytest.importorskip("torch.distributed")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, W, H, frames, out_dir):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle
    from cudapt_gb300 import layouts, scenes
    (v, t, m), cam = scenes.cornell()
    sc = oracle.Scene(v, t, m)
    rows = H // world
    r = oracle.Renderer(W, rows, 0, layouts.default_params(eye_depth_max=8, light_depth_max=8), threads=1)
    r.set_window(0, rank * rows, W, H)
    r.render(sc, cam, frames)
    band = torch.from_numpy(r.get(0).copy())
    bands = [torch.zeros_like(band) for _ in range(world)]
    dist.all_gather(bands, band)
    total = band.double().sum()
    dist.all_reduce(total)
    if rank == 0:
        np.save(os.path.join(out_dir, "img.npy"), torch.cat(bands).numpy())
        np.save(os.path.join(out_dir, "total.npy"), total.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_row_band_sharding_matches_single_rank(tmp_path, orc):
    import torch.multiprocessing as mp
    W, H, frames = 32, 32, 3
    mp.spawn(_worker, args=(2, _free_port(), W, H, frames, str(tmp_path)), nprocs=2, join=True)
    img = np.load(tmp_path / "img.npy")
    from cudapt_gb300 import layouts, scenes
    (v, t, m), cam = scenes.cornell()
    r = orc.Renderer(W, H, 0, layouts.default_params(eye_depth_max=8, light_depth_max=8), threads=2)
    r.render(orc.Scene(v, t, m), cam, frames)
    want = r.get(0)
    assert np.array_equal(img.view(np.uint32), want.view(np.uint32))
    assert abs(float(np.load(tmp_path / "total.npy")) - float(want.astype(np.float64).sum())) < 1e-6 * want.sum()
