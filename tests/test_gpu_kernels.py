"""GPU parity of the building blocks: device math, Philox, BVH traversal."""
import math
import os

import numpy as np
import pytest

from helpers import camera_rays, random_rays, scene_arrays

pytestmark = pytest.mark.gpu


def test_fmath_bitexact(gbdev, orc):
    L = gbdev._native.load()
    rng = np.random.Generator(np.random.PCG64(5))
    cases = {
        0: rng.random(1 << 18).astype(np.float32) * np.float32(2 * math.pi),
        1: rng.random(1 << 18).astype(np.float32) * np.float32(2 * math.pi),
        2: (rng.random(1 << 18) * -95.0).astype(np.float32),
        3: (rng.random(1 << 18) * 100.0).astype(np.float32),
        4: rng.random(1 << 18).astype(np.float32),
    }
    names = {0: "sin", 1: "cos", 2: "exp", 3: "sqrt_rd", 4: "pow5"}
    for which, x in cases.items():
        out = np.zeros_like(x)
        gbdev._native.check(L.gbpt_fmath(which, x.ctypes.data, len(x), out.ctypes.data))
        want = orc.fmath(names[which], x)
        assert np.array_equal(out.view(np.uint32), want.view(np.uint32)), names[which]


def test_exp_nonpositive_matches_exp(gbdev, orc):
    """The bilateral tile kernel's exponential for arguments <= 0 equals exp_p to the bit: every 67th
    float from -0 down to -90, every float within 2^-6 of the -87 cut and of the k = -126 turn, NaN."""
    L = gbdev._native.load()
    lo = np.float32(-90.0).view(np.uint32)
    bits = np.arange(0x80000000, int(lo) + 1, 67, dtype=np.uint64).astype(np.uint32)
    edges = [np.arange(int(np.float32(v - 2.0**-6).view(np.uint32)), int(np.float32(v + 2.0**-6).view(np.uint32)),
                       dtype=np.uint64).astype(np.uint32) for v in (87.0, 86.6)]
    x = np.concatenate([bits] + edges).view(np.float32)
    x = np.concatenate([-np.abs(x), np.array([0.0, np.nan], np.float32)])
    got, want = np.zeros_like(x), np.zeros_like(x)
    gbdev._native.check(L.gbpt_fmath(5, x.ctypes.data, len(x), got.ctypes.data))
    gbdev._native.check(L.gbpt_fmath(2, x.ctypes.data, len(x), want.ctypes.data))
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    finite = x[:4096 * 64]
    assert np.array_equal(got[:len(finite)].view(np.uint32), orc.fmath("exp", finite).view(np.uint32))


def test_philox_bitexact(gbdev, orc):
    L = gbdev._native.load()
    rng = np.random.Generator(np.random.PCG64(6))
    ctr = rng.integers(0, 2**32, size=(4096, 4), dtype=np.uint64).astype(np.uint32)
    out = np.zeros_like(ctr)
    gbdev._native.check(L.gbpt_philox(ctr.ctypes.data, len(ctr), 1234, 99, out.ctypes.data))
    for i in range(0, 4096, 97):
        assert np.array_equal(out[i], orc.philox(ctr[i], 1234, 99))
    # published known-answer vector (Random123, philox4x32 10 rounds)
    c = np.array([[0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344]], np.uint32)
    o = np.zeros_like(c)
    gbdev._native.check(L.gbpt_philox(c.ctypes.data, 1, 0xA4093822, 0x299F31D0, o.ctypes.data))
    assert [hex(x) for x in o[0]] == ["0xd16cfe09", "0x94fdcceb", "0x5001e420", "0x24126ea1"]


def _trace_both(gb, orc, v, t, m, rays, **kw):
    s = gb.RTScene(v, t, m).build_bvh()
    got = s.trace_rays(rays, counts=True, **kw)
    ref = orc.Scene(v, t, m).trace(rays, **{k: kw[k] for k in kw})
    return got, ref


def _assert_same_hits(got, ref):
    np.testing.assert_array_equal(got["tri"], ref["tri"])
    for k in ("t", "w", "u", "v"):
        assert np.array_equal(got[k].view(np.uint32), ref[k].view(np.uint32)), k
    np.testing.assert_array_equal(got["nodes"], ref["nodes"])
    np.testing.assert_array_equal(got["tris"], ref["tris"])


@pytest.mark.parametrize("name", ["cornell", "interior", "hall_small"])
def test_trace_bitexact_random(gbdev, orc, name):
    (v, t, m), cam = scene_arrays(name)
    rays = random_rays(v, 200_000, seed=11)
    got, ref = _trace_both(gbdev, orc, v, t, m, rays)
    assert (ref["tri"] >= 0).mean() > 0.5
    _assert_same_hits(got, ref)


@pytest.mark.parametrize("name", ["cornell", "interior", "hall_small"])
def test_trace_bitexact_camera(gbdev, orc, name):
    (v, t, m), cam = scene_arrays(name)
    rays = camera_rays(cam, 320, 240, seed=12)
    got, ref = _trace_both(gbdev, orc, v, t, m, rays)
    _assert_same_hits(got, ref)


def test_trace_bitexact_empty_children(gbdev, orc):
    """A tree with empty children keeps the reference's node order on the
    device (the right-first relayout needs every inner node to have two real
    subtrees); hits and visit counts still equal the oracle's."""
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "empty_children.npz"))
    v, t, m = g["vertices"], g["triangles"], g["materials"]
    assert orc.Scene(v, t, m).empty_children > 0
    rays = random_rays(v, 100_000, seed=15, pad=1.0)
    got, ref = _trace_both(gbdev, orc, v, t, m, rays)
    assert (ref["tri"] >= 0).mean() > 0.01
    _assert_same_hits(got, ref)
    for kw in (dict(eps=1e-4), dict(cullback=True)):
        got, ref = _trace_both(gbdev, orc, v, t, m, rays, **kw)
        _assert_same_hits(got, ref)


def test_trace_variants(gbdev, orc):
    """eps push, finite maxDist and back-face culling (CURay::IntersectTri cullback)."""
    (v, t, m), cam = scene_arrays("interior")
    rays = random_rays(v, 50_000, seed=13)
    for kw in (dict(eps=1e-4), dict(max_dist=3.0, eps=1e-4), dict(cullback=True)):
        got, ref = _trace_both(gbdev, orc, v, t, m, rays, **kw)
        _assert_same_hits(got, ref)


def test_trace_axis_aligned_and_degenerate_rays(gbdev, orc):
    """Directions with zero components exercise escapeZero (src/cudaRTCommon.cu:26-30)."""
    (v, t, m), cam = scene_arrays("cornell")
    rng = np.random.Generator(np.random.PCG64(14))
    n = 20000
    o = rng.random((n, 3)).astype(np.float32)
    d = np.zeros((n, 3), np.float32)
    ax = rng.integers(0, 3, n)
    d[np.arange(n), ax] = rng.choice([-1.0, 1.0], n)
    d[: n // 4] = 0.0  # zero direction
    rays = np.concatenate([o, d], 1)
    got, ref = _trace_both(gbdev, orc, v, t, m, rays)
    _assert_same_hits(got, ref)
