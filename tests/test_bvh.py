"""BVH build parity: the library's threaded builder against the oracle's
line-by-line restatement of src/bvhhelper.cpp (CPU only, no GPU needed)."""
import numpy as np
import pytest

from cudapt_gb300 import layouts, scenes


def _soup(n, seed, spread=10.0, size=0.5):
    rng = np.random.Generator(np.random.PCG64(seed))
    mb = scenes.MeshBuilder()
    mat = mb.add_material(layouts.material((0.5, 0.5, 0.5)))
    c = rng.random((n, 1, 3)) * spread
    mb.add_tris(c + (rng.random((n, 3, 3)) - 0.5) * size, mat)
    return mb.build()


def _compare(gb, orc, v, t, m, threads=0):
    s = gb.RTScene(v, t, m).build_bvh(threads=threads)
    b, o, order = s.bvh_export()
    ref = orc.Scene(v, t, m)
    rb, ro, rorder, _ = ref.export()
    assert ref.node_count == len(b)
    np.testing.assert_array_equal(order, rorder)
    np.testing.assert_array_equal(o, ro)
    assert np.array_equal(b.view(np.uint32), rb.view(np.uint32)), "bounds differ bitwise"
    return s, ref


@pytest.mark.parametrize("name", ["cornell", "interior"])
def test_bvh_matches_oracle_scenes(gb, orc, name):
    (v, t, m), _ = getattr(scenes, name)()
    s, ref = _compare(gb, orc, v, t, m)
    assert ref.empty_children == 0


def test_bvh_matches_oracle_hall(gb, orc):
    (v, t, m), _ = scenes.hall(boxes=300)
    _compare(gb, orc, v, t, m)


@pytest.mark.parametrize("n,seed", [(1, 0), (2, 1), (17, 2), (1000, 3), (20000, 4)])
def test_bvh_matches_oracle_soup(gb, orc, n, seed):
    v, t, m = _soup(n, seed)
    _compare(gb, orc, v, t, m)


def test_bvh_single_thread_equals_threaded(gb, orc):
    v, t, m = _soup(30000, 7)
    a = gb.RTScene(v, t, m).build_bvh(threads=1).bvh_export()
    b = gb.RTScene(v, t, m).build_bvh(threads=8).bvh_export()
    for x, y in zip(a, b):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_bvh_degenerate_inputs(gb, orc):
    # duplicated triangles (identical centroids -> leaf), a zero-area sliver,
    # axis-aligned coplanar triangles and a far-away triangle
    mb = scenes.MeshBuilder()
    mat = mb.add_material(layouts.material())
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float64)
    for _ in range(8):
        mb.add_tris(tri, mat)
    mb.add_tris(np.array([[0, 0, 0], [1, 1, 1], [2, 2, 2]]), mat)
    for k in range(16):
        mb.add_tris(tri + [k * 0.25, 0, 0], mat)
    mb.add_tris(tri + [1e4, 0, 0], mat)
    v, t, m = mb.build()
    _compare(gb, orc, v, t, m)


def test_bvh_depth_budget(gb, orc):
    v, t, m = _soup(5000, 9)
    s = gb.RTScene(v, t, m).build_bvh(max_depth=4)
    b, o, order = s.bvh_export()
    assert len(b) <= 15  # a depth-4 budget gives at most 2^4 - 1 nodes
    assert sorted(order.tolist()) == list(range(len(t)))


def test_compact_layout_invariants(gb):
    (v, t, m), _ = scenes.interior()
    s = gb.RTScene(v, t, m).build_bvh()
    b, o, order = s.bvh_export()
    n = len(b)
    inner = o[:, 1] == 0
    # inner node i: left child i+1, right child i+offset, both inside the array
    assert np.all(np.arange(n)[inner] + o[inner, 0] < n)
    # leaves partition the triangle order
    leaves = o[~inner]
    cover = np.zeros(len(t), np.int32)
    for start, cnt in leaves:
        cover[start:start + cnt] += 1
    assert np.all(cover == 1)
    # children boxes lie inside their parent box
    idx = np.nonzero(inner)[0]
    for i in idx[:2000]:
        for c in (i + 1, i + o[i, 0]):
            assert np.all(b[c, :3] >= b[i, :3]) and np.all(b[c, 3:] <= b[i, 3:])


def _empty_children_scene():
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "empty_children.npz"))
    return g["vertices"], g["triangles"], g["materials"]


def test_bvh_empty_children_fixture(gb, orc):
    """A tree with empty children ((start, 0) records the reference's walk
    enters as inner nodes, src/bvhhelper.cpp): built identically."""
    v, t, m = _empty_children_scene()
    s, ref = _compare(gb, orc, v, t, m)
    assert ref.empty_children > 0
