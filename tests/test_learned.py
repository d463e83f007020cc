"""Learned sample allocator in the renderer: tile targets on the CPU; on the
GPU the feature kernel against a numpy restatement over the renderer's own
planes, the statistics it reads (second moments, path-length counts), and
learned allocation rendering the same image as the plain allocator."""
import numpy as np
import pytest

from cudapt_gb300 import layouts, learned
from helpers import scene_arrays


def test_tile_targets():
    W, H = 20, 12  # 3 x 2 tiles, ragged
    ref = np.zeros(W * H * 3, np.float32)
    img = ref.copy().reshape(H, W, 3)
    img[:8, :8] = 1.0      # tile 0: mse 1
    img[:8, 8:16] = 0.5    # tile 1: mse 0.25
    img[8:, 16:] = 2.0     # tile 5 (4 x 4 pixels): mse 4
    t = learned.tile_targets(img.reshape(-1), ref, W, H)
    raw = 0.5 * np.log(np.array([1.0, 0.25, 0, 0, 0, 4.0]) + learned.EPS)
    np.testing.assert_allclose(t, raw - raw.mean(), rtol=1e-6, atol=1e-6)
    assert abs(t.mean()) < 1e-6


def _numpy_features(r, cam, err):
    W, H = r.width, r.height
    res = r.read_buffer(0).reshape(H, W, 3).astype(np.float64)
    n = r.read_buffer(6).reshape(H, W).astype(np.float64)
    m2 = r.read_buffer(11).reshape(H, W, 3).astype(np.float64)
    pos, nrm, dif = (r.read_buffer(k).reshape(H, W, 3).astype(np.float64) for k in (1, 2, 3))
    hist = r.read_buffer(12).reshape(-1, 8).astype(np.float64)
    e = err.reshape(H, W).astype(np.float64)
    tx, ty = (W + 7) // 8, (H + 7) // 8
    out = np.zeros((tx * ty, 24))
    cp = np.array(cam["pos"], np.float64)
    for j in range(ty):
        for i in range(tx):
            sl = (slice(j * 8, min(j * 8 + 8, H)), slice(i * 8, min(i * 8 + 8, W)))
            mu = res[sl]
            var = np.where(n[sl][..., None] > 0, np.maximum(m2[sl] - mu * mu, 0) / np.maximum(n[sl][..., None], 1), 0)
            f = out[j * tx + i]
            f[0:3] = np.log1p(np.maximum(mu.reshape(-1, 3).mean(0), 0))
            f[3:6] = np.log1p(100 * var.reshape(-1, 3).mean(0))
            f[6:9] = dif[sl].reshape(-1, 3).mean(0)
            f[9:12] = nrm[sl].reshape(-1, 3).mean(0)
            f[12] = np.log1p(np.linalg.norm(pos[sl] - cp, axis=-1).mean())
            h = hist[j * tx + i]
            f[13:21] = h / h.sum() if h.sum() > 0 else 0
            f[21] = np.log2(1 + n[sl].mean())
            f[22] = np.log1p(1000 * e[sl].mean())
            f[23] = np.log1p(1000 * e[sl].max())
    return out


@pytest.mark.gpu
def test_gpu_features_match_numpy(gbdev):
    (v, t, m), cam = scene_arrays("cornell")
    W, H = 52, 36  # ragged tiles on both axes
    s = gbdev.RTScene(v, t, m).build_bvh()
    r = gbdev.RTRenderer(W, H, layouts.MODE_BDPT_SC_ADAP_BILAT,
                         learned.adaptive_params(8, warmup_frames=2, filter_radius=3))
    r.set_mlp(None, collect=True)
    paths = 0
    for _ in range(4):
        r.render(s, cam)
        paths += r.last_stats["paths"]
    f = r.features()
    assert f.shape == (7 * 5, 24)
    hist = r.read_buffer(12)
    # every camera path of the 4 frames (2 uniform frames of W*H, 2 budgeted) ended exactly once
    assert hist.sum() == paths and paths > 2 * W * H
    m2, mu = r.read_buffer(11), r.read_buffer(0)
    assert np.all(m2 >= mu * mu * (1 - 1e-5) - 1e-7)  # E[x^2] >= E[x]^2
    want = _numpy_features(r, cam, r.read_buffer(5))
    np.testing.assert_allclose(f, want, rtol=2e-4, atol=2e-5)


@pytest.mark.gpu
def test_gpu_learned_allocation_renders_same_image(gbdev):
    """The network changes where samples go, not what converges: images of
    the plain allocator, of a network whose output is constant (equal budget
    per tile) and of a random network all approach the same long plain
    render, with errors of the same size."""
    from cudapt_gb300.mlp import MLP
    from oracle import mlp_ref
    (v, t, m), cam = scene_arrays("cornell")
    W, H = 48, 48
    s = gbdev.RTScene(v, t, m).build_bvh()
    p = learned.adaptive_params(8, warmup_frames=2, filter_radius=3)
    ref = learned.converged(gbdev, s, cam, W, H, 2048, depth=8)
    flat = mlp_ref.init(4)
    flat[-65:] = 0.0  # w3 = 0, b3 = 0: every tile gets weight exp(0)
    nets = {"plain": None, "flat": MLP(params=flat.astype(np.float32)), "random": MLP(seed=3)}
    err, counts = {}, {}
    for name, mlp in nets.items():
        r = gbdev.RTRenderer(W, H, layouts.MODE_BDPT_SC_ADAP_BILAT, p)
        r.set_mlp(mlp)
        for _ in range(40):
            img = r.render(s, cam)
            assert r.last_stats["paths"] <= W * H
        counts[name] = r.read_buffer(6).copy()
        err[name] = float(np.sqrt(np.mean((img.astype(np.float64) - ref) ** 2)))
        assert abs(img.mean() - ref.mean()) <= 0.08 * ref.mean(), (name, img.mean(), ref.mean())
    assert not np.array_equal(counts["plain"], counts["random"])  # the allocation differs
    assert not np.array_equal(counts["plain"], counts["flat"])
    for name in ("flat", "random"):
        assert err[name] <= 2.5 * err["plain"], err


@pytest.mark.gpu
def test_gpu_training_on_rendered_tiles(gbdev):
    """Samples from three small hall scenes: the trained network predicts a
    held-out scene's tile errors better than a constant and better than the
    plain heuristic's own tile error (a least-squares line on that feature,
    fitted to the same training tiles).  The equal-time RMSE of the learned
    allocation itself does not beat the plain allocator on these scenes
    (tests/experiments/learned_sampler.py), so no test asserts that."""
    Xs, Ys = [], []
    for seed in (1, 2, 3, 21):
        X, Y = learned.samples_for_scene(gbdev, seed, width=160, height=96, snapshots=(2, 5, 8), conv_frames=256,
                                         boxes=120, warmup=2)
        Xs.append(X)
        Ys.append(Y)
    Xt, Yt = np.concatenate(Xs[:3]), np.concatenate(Ys[:3])
    net, losses = learned.train(Xt, Yt, steps=600, batch=1024, lr=3e-3)
    assert losses[-20:].mean() < 0.7 * losses[:5].mean()
    pred = net.forward(Xs[3])
    pred -= pred.mean()
    A = np.stack([Xt[:, 22], np.ones(len(Xt))], 1)
    coef = np.linalg.lstsq(A, Yt, rcond=None)[0]
    line = np.stack([Xs[3][:, 22], np.ones(len(Xs[3]))], 1) @ coef
    line -= line.mean()
    mse_net, mse_line, mse_const = (float(np.mean((x - Ys[3]) ** 2)) for x in (pred, line, 0.0))
    assert mse_net < 0.9 * mse_const, (mse_net, mse_const)
    assert mse_net < mse_line, (mse_net, mse_line)
