"""The float thresholds of cudapt_gb300/csrc/gbpt_math.cuh give the same
answers as the reference's comparisons against double literals, for every
float around each threshold (the comparisons are monotonic, so the window
around the switch point decides all floats)."""
import re
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _consts():
    src = open(os.path.join(ROOT, "cudapt_gb300", "csrc", "gbpt_math.cuh")).read()
    out = {}
    for name, val in re.findall(r"constexpr float (k\w+) = ([0-9a-fx.p+-]+)f;", src):
        out[name] = np.float32(float.fromhex(val))
    return out


def _window(center, n=1 << 18):
    c = np.float32(center).view(np.uint32).astype(np.int64)
    bits = np.arange(c - n, c + n, dtype=np.int64).astype(np.uint32)
    return bits.view(np.float32)


def test_thresholds_equal_double_comparisons():
    k = _consts()
    f = _window(1e-9)
    assert np.array_equal(f.astype(np.float64) < 1e-9, f < k["kLtEps9"])
    assert np.array_equal(f.astype(np.float64) > 1e-9, f > k["kGtEps9"])
    f = _window(1e-4)
    assert np.array_equal(f.astype(np.float64) < 1e-4, f < k["kLtEps4"])
    f = _window(1.0 - 1e-4)
    assert np.array_equal(f.astype(np.float64) + 1e-4 > 1.0, f >= k["kProbOne"])
    f = _window(0.1)
    assert np.array_equal(f.astype(np.float64) > 0.1, f >= k["kPointOne"])
    f = _window(1e-5)
    assert np.array_equal(f.astype(np.float64) > 1e-5, f > k["kFltEps"])


def test_rounded_literals():
    k = _consts()
    import math
    assert k["kInf"] == np.float32(1e20) and k["kBias"] == np.float32(1e-4)
    assert k["kPi"] == np.float32(math.pi) and k["kInvPi"] == np.float32(1 / math.pi)
    assert k["kTwoPi"] == np.float32(2 * math.pi) and k["kF0Spec"] == np.float32(0.08)
    assert k["kEps9f"] == np.float32(1e-9)


def test_transcendentals_accuracy(orc):
    x = np.linspace(-20.0, 20.0, 400001).astype(np.float32)
    s, c = orc.fmath("sin", x), orc.fmath("cos", x)
    assert np.abs(s - np.sin(x.astype(np.float64))).max() < 4e-7
    assert np.abs(c - np.cos(x.astype(np.float64))).max() < 4e-7
    y = np.linspace(-86.9, 10.0, 400001).astype(np.float32)
    e = orc.fmath("exp", y).astype(np.float64)
    ref = np.exp(y.astype(np.float64))
    assert (np.abs(e - ref) / ref).max() < 3e-7
    assert orc.fmath("exp", np.array([-87.5, -200.0], np.float32)).tolist() == [0.0, 0.0]
    r = np.abs(np.random.default_rng(0).normal(size=100000)).astype(np.float32) * 100
    q = orc.fmath("sqrt_rd", r).astype(np.float64)
    assert np.all(q * q <= r.astype(np.float64))                        # never rounds up
    nxt = np.nextafter(q.astype(np.float32), np.float32(np.inf)).astype(np.float64)
    assert np.all(nxt * nxt > r.astype(np.float64))                     # and is the largest such float
