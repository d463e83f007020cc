"""Image files and RMSE experiments (src/cudapt.cpp:482-619, 840-997,
src/hdrhelper.cpp): file formats round-trip on the CPU; the GPU conversions
and the RMSE harness against numpy restatements of the reference's loops."""
import numpy as np
import pytest

from cudapt_gb300 import imageio
from helpers import scene_arrays


def test_png_round_trip(tmp_path):
    rng = np.random.Generator(np.random.PCG64(3))
    a = rng.integers(0, 256, (13, 21, 4), dtype=np.uint8)
    imageio.write_png(tmp_path / "a.png", a, 21, 13)
    b, w, h = imageio.read_png(tmp_path / "a.png")
    assert (w, h) == (21, 13) and np.array_equal(a, b)


def test_bmp_round_trip(tmp_path):
    rng = np.random.Generator(np.random.PCG64(4))
    a = rng.integers(0, 256, (7, 11, 3), dtype=np.uint8)  # 33-byte rows: padded to 36
    imageio.write_bmp(tmp_path / "a.bmp", a, 11, 7)
    b, w, h = imageio.read_bmp(tmp_path / "a.bmp")
    assert (w, h) == (11, 7) and np.array_equal(a, b)
    assert (tmp_path / "a.bmp").stat().st_size == 54 + 7 * 36


@pytest.mark.parametrize("rle", [True, False])
def test_rgbe_round_trip(tmp_path, rle):
    rng = np.random.Generator(np.random.PCG64(5))
    W, H = 40, 9
    img = (rng.random(W * H * 3) * 50.0).astype(np.float32)
    img[:30] = 0.0                       # zero pixels (exponent 0)
    img[300:420] = 2.5                   # a run for the RLE coder
    imageio.write_rgbe(tmp_path / "a.hdr", img, W, H, rle=rle)
    back, w, h = imageio.read_rgbe(tmp_path / "a.hdr")
    assert (w, h) == (W, H)
    # RGBE keeps 8 mantissa bits of the largest channel: relative error <= 2^-8 of that channel
    big = np.repeat(img.reshape(-1, 3).max(1), 3)
    assert np.all(np.abs(back - img) <= big * 2.0 ** -7 + 1e-30)
    assert np.all(back[:30] == 0.0)
    # bytes equal the published conversion (frexp mantissa * 256 / v, truncated)
    q = imageio.float_to_rgbe(np.array([[1.0, 0.5, 0.25], [0.0, 0.0, 0.0], [3.0, 7.0, 1e-3]], np.float32))
    assert q.tolist() == [[128, 64, 32, 129], [0, 0, 0, 0], [96, 224, 0, 131]]


def test_rgbe_rle_smaller_on_flat_image(tmp_path):
    img = np.full(64 * 8 * 3, 0.75, np.float32)
    imageio.write_rgbe(tmp_path / "r.hdr", img, 64, 8, rle=True)
    imageio.write_rgbe(tmp_path / "f.hdr", img, 64, 8, rle=False)
    assert (tmp_path / "r.hdr").stat().st_size < (tmp_path / "f.hdr").stat().st_size / 4
    a, _, _ = imageio.read_rgbe(tmp_path / "r.hdr")
    b, _, _ = imageio.read_rgbe(tmp_path / "f.hdr")
    assert np.array_equal(a, b)


def _ref_bytes(rgb, W, H, exposure, kind, ref=None):
    """numpy restatement of the reference's export loops (float32 arithmetic)."""
    c = np.asarray(rgb, np.float32).reshape(H, W, 3)[::-1]
    if kind == 1:
        d = c - np.asarray(ref, np.float32).reshape(H, W, 3)[::-1]
        m = np.clip((d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1] + d[..., 2] * d[..., 2]) / np.float32(3),
                    0, 1).astype(np.float32)
        x = np.repeat(m[..., None], 3, axis=2)
    else:
        x = np.clip(c, 0, 1).astype(np.float32)
        if kind == 0:
            x = (np.float32(1) - np.exp(-x * np.float32(exposure))).astype(np.float32)
            x = np.power(x, np.float32(1 / 2.2)).astype(np.float32)
    return (x * np.float32(255)).astype(np.uint8)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", [0, 1, 2])
def test_gpu_tonemap_matches_reference_loop(gbdev, kind):
    rng = np.random.Generator(np.random.PCG64(6 + kind))
    W, H = 37, 23
    img = (rng.random(W * H * 3) * 3.0 - 0.2).astype(np.float32)
    ref = (rng.random(W * H * 3) * 2.0).astype(np.float32)
    got = imageio.tonemap(img, W, H, 1.7, kind, ref)
    want = _ref_bytes(img, W, H, 1.7, kind, ref)
    assert np.all(got[..., 3] == 255)
    diff = np.abs(got[..., :3].astype(int) - want.astype(int))
    assert diff.max() <= 1 and np.mean(diff > 0) <= 0.01  # exp/pow may round differently by one byte


@pytest.mark.gpu
def test_gpu_rmse_and_harness(gbdev, tmp_path):
    rng = np.random.Generator(np.random.PCG64(9))
    a = rng.random(300001).astype(np.float32)
    b = rng.random(300001).astype(np.float32)
    want = np.sqrt(np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2))
    assert abs(imageio.rmse(a, b) - want) <= 1e-12 * want

    from cudapt_gb300 import experiment
    (v, t, m), cam = scene_arrays("cornell")
    s = gbdev.RTScene(v, t, m).build_bvh()
    W = H = 48
    r = gbdev.RTRenderer(W, H, 0, gbdev.default_params(eye_depth_max=6, light_depth_max=6))
    conv = experiment.capture_converged(r, s, cam, 64)
    assert r.rmse(conv) == 0.0
    rows = experiment.collect(r, s, cam, conv, interval_s=1e-4, n_points=6, csv_path=tmp_path / "d.csv")
    assert len(rows) == 6 and [n for _, n, _ in rows] == sorted(n for _, n, _ in rows)
    assert rows[-1][2] < rows[0][2]  # error falls as frames accumulate
    lines = (tmp_path / "d.csv").read_text().splitlines()
    assert len(lines) == 6 and len(lines[0].split(", ")) == 3
    img = r.GetResult().copy()
    host = np.sqrt(np.mean((img.astype(np.float64) - conv.astype(np.float64)) ** 2))
    assert abs(r.rmse(conv) - host) <= 1e-9 * max(host, 1e-12)
    s_, n_, e_ = experiment.until(r, s, cam, conv, frames=5)
    assert n_ == 5 and e_ > 0
    _, n2, e2 = experiment.until(r, s, cam, conv, rmse_limit=rows[2][2])
    assert e2 <= rows[2][2]
    imageio.save_result_png(tmp_path / "r.png", img, W, H)
    back, w, h = imageio.read_png(tmp_path / "r.png")
    assert np.array_equal(back, imageio.tonemap(img, W, H))
