"""Row-band sharding of one image across ranks (world_size 2, gloo, CPU).

Pixels are independent and every path's random numbers are fixed by its
global pixel id, so each rank renders the band of rows that
cudapt_gb300.sharding assigns it and the gathered bands equal the
single-process image bit for bit; the light-vertex cache is replicated (same
key and frame on every rank).  The ranks render with the oracle here (CPU
ranks, no GPU); on a GPU the library renders the same bands through
RTRenderer.set_window (tests/test_gpu_render.py::test_windows_assemble_the_image).
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
    from cudapt_gb300 import layouts, scenes, sharding
    (v, t, m), cam = scenes.cornell()
    sc = oracle.Scene(v, t, m)
    y0, rows = sharding.shard_rows(H, world, rank)
    r = oracle.Renderer(W, rows, 0, layouts.default_params(eye_depth_max=8, light_depth_max=8), threads=1)
    r.set_window(0, y0, W, H)
    r.render(sc, cam, frames)
    band = torch.from_numpy(r.get(0).copy())
    # ragged bands: gather padded to the largest, then cut each to its rows
    most = sharding.shard_rows(H, world, 0)[1] * W * 3
    padded = torch.zeros(most, dtype=band.dtype)
    padded[: band.numel()] = band
    bands = [torch.zeros_like(padded) for _ in range(world)]
    dist.all_gather(bands, padded)
    total = band.double().sum()
    dist.all_reduce(total)
    if rank == 0:
        parts = [bands[k][: sharding.shard_rows(H, world, k)[1] * W * 3].numpy() for k in range(world)]
        np.save(os.path.join(out_dir, "img.npy"), sharding.assemble(parts, W))
        np.save(os.path.join(out_dir, "total.npy"), total.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_row_band_sharding_matches_single_rank(tmp_path, orc):
    import torch.multiprocessing as mp
    W, H, frames = 32, 33, 3  # 33 rows: ragged bands (17 + 16)
    mp.spawn(_worker, args=(2, _free_port(), W, H, frames, str(tmp_path)), nprocs=2, join=True)
    img = np.load(tmp_path / "img.npy")
    from cudapt_gb300 import layouts, scenes
    (v, t, m), cam = scenes.cornell()
    r = orc.Renderer(W, H, 0, layouts.default_params(eye_depth_max=8, light_depth_max=8), threads=2)
    r.render(orc.Scene(v, t, m), cam, frames)
    want = r.get(0)
    assert np.array_equal(img.view(np.uint32), want.view(np.uint32))
    assert abs(float(np.load(tmp_path / "total.npy")) - float(want.astype(np.float64).sum())) < 1e-6 * want.sum()


def test_shard_rows_cover_the_image():
    from cudapt_gb300 import sharding
    for H in (1, 7, 33, 720):
        for world in (1, 2, 3, 8):
            parts = [sharding.shard_rows(H, world, k) for k in range(world)]
            assert parts[0][0] == 0 and sum(r for _, r in parts) == H
            assert all(parts[k][0] + parts[k][1] == parts[k + 1][0] for k in range(world - 1))
            assert max(r for _, r in parts) - min(r for _, r in parts) <= 1
    with pytest.raises(ValueError):
        sharding.shard_rows(10, 2, 2)


def _sync_worker(rank, world, port, out_dir):
    import sys
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    s = bench.RankSync(world)
    s.barrier()
    m = s.max(10.0 + rank)  # each rank's time; the job's is the slowest
    s.barrier()
    with open(os.path.join(out_dir, f"max{rank}.txt"), "w") as f:
        f.write(repr(m))
    dist.destroy_process_group()


def test_bench_rank_sync_takes_the_slowest_rank(tmp_path):
    """bench.py's replicas time the job by the slowest rank (barriers around
    the timed steps, max over ranks), here with two gloo ranks on the CPU."""
    import torch.multiprocessing as mp
    mp.spawn(_sync_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    for r in (0, 1):
        assert float((tmp_path / f"max{r}.txt").read_text()) == 11.0
