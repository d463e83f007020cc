"""TEST INFRASTRUCTURE ONLY -- CPU oracle of the learned sample allocator.

A restatement, in float64 numpy, of the MLP the CUDA kernels train and run
(csrc/mlp.cu): 24 -> 64 -> 64 -> 1 with GELU (the erf form,
0.5 x (1 + erf(x / sqrt 2))), BF16 weights and BF16 layer inputs, every
product accumulated in FP32 on the GPU (float64 here), mean-squared-error
loss and Adam (Kingma & Ba, ICLR 2015: beta1 0.9, beta2 0.999, eps 1e-8,
bias-corrected).  The reference has no learned sampler (CudaPT links FANN
but never calls it), so this oracle follows the method's published maths;
the GPU's gradients are checked against it and against finite differences.

The rounding points follow the kernels exactly: inputs X, weights W1, W2,
w3, hidden activations H1 and the backpropagated dZ2, dZ1 are rounded to
BF16 (round to nearest even) where the kernels feed them to the tensor
cores; biases, pre-activations, H2, y and all accumulators stay wide.
"""
import math

import numpy as np

N_IN, N_IN_PAD, N_HID = 24, 32, 64
# parameter vector layout (fp32 master copy)
SHAPES = [("w1", (N_HID, N_IN)), ("b1", (N_HID,)), ("w2", (N_HID, N_HID)), ("b2", (N_HID,)), ("w3", (N_HID,)),
          ("b3", (1,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)  # 5825


def unpack(theta):
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = np.asarray(theta[o:o + n], np.float64).reshape(shp)
        o += n
    return out


def pack(p):
    return np.concatenate([np.asarray(p[name], np.float64).reshape(-1) for name, _ in SHAPES])


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.asarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    r = np.where(np.isnan(a), u | 0x400000, r)
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


_erf = np.vectorize(math.erf)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def forward(theta, x, keep=False, exact=False):
    """exact: no BF16 rounding anywhere (the smooth function finite differences can check)."""
    p = unpack(theta)
    r = (lambda a: np.asarray(a, np.float64)) if exact else bf16
    X = r(np.asarray(x, np.float64 if exact else np.float32))
    W1, W2, w3 = r(p["w1"]), r(p["w2"]), r(p["w3"])
    Z1 = X @ W1.T + p["b1"]
    H1 = r(gelu(Z1))
    Z2 = H1 @ W2.T + p["b2"]
    H2 = gelu(Z2)
    y = H2 @ w3 + p["b3"][0]
    if keep:
        return y, dict(X=X, W1=W1, W2=W2, w3=w3, Z1=Z1, H1=H1, Z2=Z2, H2=H2, r=r)
    return y


def loss(theta, x, t, exact=False):
    y = forward(theta, x, exact=exact)
    return float(np.mean((y - np.asarray(t, np.float64)) ** 2))


def gradients(theta, x, t, exact=False):
    """Gradient of the mean squared error with the kernels' BF16 rounding points
    (exact: of the unrounded network)."""
    y, c = forward(theta, x, keep=True, exact=exact)
    r = c["r"]
    n = len(y)
    dy = 2.0 * (y - np.asarray(t, np.float64)) / n
    g = {}
    g["w3"] = c["H2"].T @ dy
    g["b3"] = np.array([dy.sum()])
    dZ2 = np.outer(dy, c["w3"]) * gelu_grad(c["Z2"])
    dZ2b = r(dZ2)
    g["w2"] = dZ2b.T @ c["H1"]
    g["b2"] = dZ2.sum(0)
    dH1 = dZ2b @ c["W2"]
    dZ1 = dH1 * gelu_grad(c["Z1"])
    dZ1b = r(dZ1)
    g["w1"] = dZ1b.T @ c["X"]
    g["b1"] = dZ1.sum(0)
    return pack(g)


def adam_step(theta, m, v, grad, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update; `step` counts from 1.  Returns new (theta, m, v)."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return theta - lr * mh / (np.sqrt(vh) + eps), m, v


def init(seed):
    """He-uniform weights (bound sqrt(6 / fan_in)), zero biases: numpy's PCG64 here; the library
    draws its own (gbpt_mlp_create) and the tests pass weights explicitly."""
    rng = np.random.Generator(np.random.PCG64(seed))
    p = {}
    for name, shp in SHAPES:
        if name.startswith("w"):
            fan = shp[-1] if len(shp) == 2 else N_HID
            p[name] = rng.uniform(-1, 1, shp) * math.sqrt(6.0 / fan)
        else:
            p[name] = np.zeros(shp)
    return pack(p)
