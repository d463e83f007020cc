"""Learned sample allocator: the MLP oracle (float64 numpy restatement with
the kernels' BF16 rounding points) checked against finite differences, and
the tcgen05 kernels (forward, gradients, Adam, training) against the oracle."""
import numpy as np
import pytest

from oracle import mlp_ref


def _data(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    x = rng.normal(size=(n, 24)).astype(np.float32)
    t = (np.sin(x[:, :4].sum(1)) + 0.3 * x[:, 5] * x[:, 7]).astype(np.float32)
    return x, t


def test_oracle_gradients_match_finite_differences():
    x, t = _data(37, 1)
    th = mlp_ref.init(3)
    th[mlp_ref.N_PARAMS - 1] = 0.2
    g = mlp_ref.gradients(th, x, t, exact=True)
    rng = np.random.Generator(np.random.PCG64(2))
    idx = np.concatenate([rng.choice(mlp_ref.N_PARAMS, 60, replace=False), [mlp_ref.N_PARAMS - 1]])
    h = 1e-6
    for i in idx:
        e = np.zeros_like(th)
        e[i] = h
        fd = (mlp_ref.loss(th + e, x, t, exact=True) - mlp_ref.loss(th - e, x, t, exact=True)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_oracle_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0, 65504.0], np.float32)
    r = mlp_ref.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0  # halfway: to even
    assert r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-12 and r[4] == 0.0 and r[5] == 65536.0


def test_oracle_adam_first_step_moves_by_lr():
    th = np.zeros(4)
    g = np.array([1.0, -2.0, 0.5, 0.0])
    new, m, v = mlp_ref.adam_step(th, np.zeros(4), np.zeros(4), g, 1, lr=1e-3)
    np.testing.assert_allclose(new[:3], -1e-3 * np.sign(g[:3]), rtol=1e-6)
    assert new[3] == 0.0


@pytest.mark.gpu
def test_gpu_mlp_forward_matches_oracle(gbdev):
    from cudapt_gb300.mlp import MLP
    x, _ = _data(1000, 5)  # 8 CTAs, the last one partly filled
    th = mlp_ref.init(7).astype(np.float32)
    th[mlp_ref.N_PARAMS - 65:mlp_ref.N_PARAMS - 1] *= 0.5
    net = MLP(params=th)
    y = net.forward(x)
    want = mlp_ref.forward(th.astype(np.float64), x)
    scale = np.abs(want).max()
    np.testing.assert_allclose(y, want, rtol=2e-3, atol=2e-3 * scale)


@pytest.mark.gpu
def test_gpu_mlp_gradients_match_oracle(gbdev):
    from cudapt_gb300.mlp import MLP
    x, t = _data(777, 6)
    th = mlp_ref.init(8).astype(np.float32)
    net = MLP(params=th)
    g, loss = net.gradients(x, t)
    want = mlp_ref.gradients(th.astype(np.float64), x, t)
    assert abs(loss - mlp_ref.loss(th.astype(np.float64), x, t)) <= 1e-3 * loss
    for name, (a, b) in zip(("w1", "b1", "w2", "b2", "w3", "b3"),
                            ((0, 1536), (1536, 1600), (1600, 5696), (5696, 5760), (5760, 5824), (5824, 5825))):
        gg, ww = g[a:b].astype(np.float64), want[a:b]
        cos = gg @ ww / (np.linalg.norm(gg) * np.linalg.norm(ww) + 1e-30)
        assert cos > 0.9999, (name, cos)
        np.testing.assert_allclose(gg, ww, rtol=0.05, atol=0.02 * np.abs(ww).max(), err_msg=name)


@pytest.mark.gpu
def test_gpu_mlp_adam_step_and_training(gbdev):
    from cudapt_gb300.mlp import MLP
    x, t = _data(4096, 9)
    th = mlp_ref.init(10).astype(np.float32)
    net = MLP(params=th)
    g, _ = net.gradients(x, t)
    l0 = net.train_step(x, t, lr=1e-3)
    new = net.params.astype(np.float64)
    want, _, _ = mlp_ref.adam_step(th.astype(np.float64), np.zeros(len(th)), np.zeros(len(th)),
                                   g.astype(np.float64), 1, lr=1e-3)
    np.testing.assert_allclose(new, want, rtol=1e-5, atol=1e-6)
    for _ in range(300):
        loss = net.train_step(x, t, lr=3e-3)
    assert loss < 0.3 * l0, (l0, loss)
    xv, tv = _data(2048, 11)
    yv = net.forward(xv)
    assert np.mean((yv - tv) ** 2) < 0.5 * np.mean((tv - tv.mean()) ** 2)
