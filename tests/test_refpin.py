"""The oracle pinned to the reference's own code: src/bvhhelper.cpp and
src/cudaRTCommon.cu compiled from the CudaPT checkout (oracle/refpin) and
compared with the oracle's restatement and the library's builder, to the
bit.  Runs where the checkout is present (the build container); the
fixtures it produces (tests/golden/make_refpin_golden.py) carry the pin to
the GPU tests elsewhere."""
import numpy as np
import pytest

from cudapt_gb300 import layouts, scenes
from helpers import assert_bits_equal, camera_rays, random_rays, scene_arrays


@pytest.fixture(scope="module")
def ref():
    from oracle import refpin
    if not refpin.build():
        pytest.skip("reference checkout absent: the pin library cannot be built here")
    return refpin


def _soup(n, seed, spread=10.0, size=0.5):
    rng = np.random.Generator(np.random.PCG64(seed))
    mb = scenes.MeshBuilder()
    mat = mb.add_material(layouts.material((0.5, 0.5, 0.5)))
    c = rng.random((n, 1, 3)) * spread
    mb.add_tris(c + (rng.random((n, 3, 3)) - 0.5) * size, mat)
    return mb.build()


def _degenerate():
    mb = scenes.MeshBuilder()
    mat = mb.add_material(layouts.material())
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float64)
    for _ in range(8):
        mb.add_tris(tri, mat)
    mb.add_tris(np.array([[0, 0, 0], [1, 1, 1], [2, 2, 2]]), mat)
    for k in range(16):
        mb.add_tris(tri + [k * 0.25, 0, 0], mat)
    mb.add_tris(tri + [1e4, 0, 0], mat)
    return mb.build()


def _scenes():
    out = {name: scene_arrays(name)[0] for name in ("cornell", "interior")}
    out["hall_small"] = scenes.hall(boxes=200)[0]
    out["soup_2"] = _soup(2, 1)
    out["soup_20000"] = _soup(20000, 4)
    out["degenerate"] = _degenerate()
    d = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "empty_children.npz"))
    out["empty_children"] = (d["vertices"], d["triangles"], d["materials"])
    return out


SCENES = _scenes()


@pytest.mark.parametrize("name", sorted(SCENES))
def test_bvh_build_equals_reference(ref, orc, gb, name):
    """CreateBVH + InitialCompactBVH of the reference against the oracle and
    the library's threaded builder: bounds, child/leaf words, triangle order
    and the device intersection records (p0, p1-p0, p2-p0)."""
    v, t, m = SCENES[name]
    rs = ref.RefScene(v, t)
    rb, ro, rorder, risect = rs.export()
    ob, oo, oorder, oisect = orc.Scene(v, t, m).export()
    assert_bits_equal(ob, rb, "oracle bounds")
    assert_bits_equal(oo, ro, "oracle offsets")
    assert_bits_equal(oorder, rorder, "oracle order")
    assert_bits_equal(oisect, risect, "oracle intersection records")
    lb, lo, lorder = gb.RTScene(v, t, m).build_bvh().bvh_export()
    assert_bits_equal(lb, rb, "library bounds")
    assert_bits_equal(lo, ro, "library offsets")
    assert_bits_equal(lorder, rorder, "library order")


@pytest.mark.parametrize("name", ["cornell", "interior", "hall_small", "degenerate", "empty_children"])
def test_trace_primitive_equals_reference(ref, orc, name):
    """TracePrimitive of the reference (device arithmetic: IEEE intrinsics,
    round-down square root) against the oracle on random and camera rays,
    for the closest-hit epsilon, the shadow epsilon with a distance cap and
    back-face culling."""
    v, t, m = SCENES[name]
    rs = ref.RefScene(v, t)
    osc = orc.Scene(v, t, m)
    rays = random_rays(v, 20000, 11)
    if name in ("cornell", "interior"):
        cam = scene_arrays(name)[1]
        rays = np.concatenate([rays, camera_rays(cam, 96, 64, 3)])
    for max_dist, eps, cull in ((1e20, 1e-9, False), (1e20, 1e-9, True), (7.5, 1e-4, False)):
        a = rs.trace(rays, max_dist=max_dist, eps=eps, cullback=cull)
        b = osc.trace(rays, max_dist=max_dist, eps=eps, cullback=cull)
        for k in ("t", "tri", "w", "u", "v"):
            assert_bits_equal(b[k], a[k], f"{name} {k} (max {max_dist}, eps {eps}, cull {cull})")


def _adversarial_rays(rng, n):
    o = (rng.random((n, 3)) * 4 - 2).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d.astype(np.float32)
    k = n // 4
    d[:k, rng.integers(0, 3, k)] = 0.0                  # axis-parallel: escapeZero of a zero component
    d[k:2 * k, 0] = np.float32(1e-10)                    # components below M_EPSILON
    d[2 * k:3 * k] = np.round(d[2 * k:3 * k] * 2) / 2    # exact, repeated directions
    return o, d


def test_intersect_aabb_equals_reference(ref, orc):
    rng = np.random.Generator(np.random.PCG64(31))
    n = 200000
    o, d = _adversarial_rays(rng, n)
    lo = (rng.random((n, 3)) * 2 - 1).astype(np.float32)
    hi = lo + (rng.random((n, 3)) * rng.choice([0.0, 1e-7, 1.0], (n, 1))).astype(np.float32)  # flat and thin boxes
    o[: n // 8] = (lo[: n // 8] + hi[: n // 8]) / 2                                         # origins inside
    cases = np.concatenate([o, d, lo, hi], 1)
    assert_bits_equal(orc.intersect_aabb(cases), ref.intersect_aabb(cases), "IntersectAABB")


def test_intersect_tri_equals_reference(ref, orc):
    rng = np.random.Generator(np.random.PCG64(32))
    n = 200000
    o, d = _adversarial_rays(rng, n)
    p0 = (rng.random((n, 3)) * 2 - 1).astype(np.float32)
    e0 = (rng.normal(size=(n, 3)) * rng.choice([1e-6, 0.1, 1.0], (n, 1))).astype(np.float32)
    e1 = (rng.normal(size=(n, 3)) * rng.choice([1e-6, 0.1, 1.0], (n, 1))).astype(np.float32)
    e1[: n // 10] = e0[: n // 10] * np.float32(2.0)     # degenerate (zero area)
    aim = p0 + 0.3 * e0 + 0.3 * e1                        # half the rays aimed at the triangle
    half = n // 2
    dd = aim[half:] - o[half:]
    d[half:] = (dd / np.linalg.norm(dd, axis=1, keepdims=True)).astype(np.float32)
    cases = np.concatenate([o, d, p0, e0, e1], 1)
    for eps, cull in ((1e-9, True), (1e-9, False), (1e-4, False)):
        a = ref.intersect_tri(cases, eps=eps, cullback=cull)
        b = orc.intersect_tri(cases, eps=eps, cullback=cull)
        assert_bits_equal(b, a, f"IntersectTri eps {eps} cull {cull}")
        assert np.mean(a[:, 0] < 1e19) > 0.1  # enough hits to mean something
