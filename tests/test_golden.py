"""Golden fixtures (tests/golden/, made by tests/golden/make_golden.py from the
reference's own cornell_box_with_sphere.obj asset and the procedural Cornell
box).  CPU tests pin the oracle and the library's BVH builder to them; the GPU
test pins the kernels."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# Philox4x32-10 known-answer vectors published with Random123 (kat_vectors).
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


def _load(name):
    return np.load(os.path.join(GOLD, name))


def test_philox_known_answers(orc):
    for ctr, key, want in PHILOX_KAT:
        assert tuple(int(x) for x in orc.philox(ctr, *key)) == want


def test_obj_bvh_and_hits_oracle(orc):
    d = _load("obj_cornell.npz")
    sc = orc.Scene(d["vertices"], d["triangles"], d["materials"])
    b, o, order, _ = sc.export()
    assert np.array_equal(b.view(np.uint32), d["bounds"].view(np.uint32))
    assert np.array_equal(o, d["off"]) and np.array_equal(order, d["order"])
    h = sc.trace(d["rays"], eps=1e-4)
    for k in ("t", "tri", "w", "u", "v", "nodes", "tris"):
        assert np.array_equal(h[k].view(np.uint32), d["hit_" + k].view(np.uint32)), k


def test_obj_bvh_library_builder(gb):
    d = _load("obj_cornell.npz")
    s = gb.RTScene(d["vertices"], d["triangles"], d["materials"]).build_bvh()
    b, o, order = s.bvh_export()
    assert np.array_equal(b.view(np.uint32), d["bounds"].view(np.uint32))
    assert np.array_equal(o, d["off"]) and np.array_equal(order, d["order"])


def test_cornell_frames_oracle(orc):
    d = _load("cornell_frames.npz")
    sc = orc.Scene(d["vertices"], d["triangles"], d["materials"])
    cam = dict(pos=d["cam"][0:3], dir=d["cam"][3:6], up=d["cam"][6:9], fov=float(d["cam"][9]))
    r = orc.Renderer(24, 24, 0, d["params"], threads=2)
    for f in range(3):
        r.render(sc, cam, 1)
        assert np.array_equal(r.get(0).view(np.uint32), d["frames"][f].view(np.uint32)), f
        if f == 0:
            assert np.array_equal(r.light_cache().view(np.uint32), d["cache"].view(np.uint32))


@pytest.mark.gpu
def test_golden_gpu(gbdev):
    d = _load("obj_cornell.npz")
    s = gbdev.RTScene(d["vertices"], d["triangles"], d["materials"]).build_bvh()
    h = s.trace_rays(d["rays"], eps=1e-4, counts=True)
    for k in ("t", "tri", "w", "u", "v", "nodes", "tris"):
        assert np.array_equal(h[k].view(np.uint32), d["hit_" + k].view(np.uint32)), k
    d = _load("cornell_frames.npz")
    s = gbdev.RTScene(d["vertices"], d["triangles"], d["materials"]).build_bvh()
    cam = dict(pos=d["cam"][0:3], dir=d["cam"][3:6], up=d["cam"][6:9], fov=float(d["cam"][9]))
    r = gbdev.RTRenderer(24, 24, 0, d["params"])
    for f in range(3):
        img = r.render(s, cam)
        assert np.array_equal(img.view(np.uint32), d["frames"][f].view(np.uint32)), f
    assert np.array_equal(r.read_buffer(6), d["sampleN"])


# ---- fixtures written from the reference's own code (make_refpin_golden.py) ----

def _refpin_scenes():
    from cudapt_gb300 import layouts
    d = _load("refpin_traces.npz")
    for name in d["names"]:
        name = str(name)
        pos, idx = d[f"{name}_pos"], d[f"{name}_idx"]
        v = np.zeros(len(pos), layouts.VERTEX)
        v["pos"] = pos
        t = np.zeros(len(idx), layouts.TRIANGLE)
        t["v0"], t["v1"], t["v2"] = idx[:, 0], idx[:, 1], idx[:, 2]
        m = np.zeros(1, layouts.MATERIAL)
        m[0] = layouts.material()
        yield name, (v, t, m), d


def test_refpin_fixture_oracle(orc):
    """The oracle's BVH and TracePrimitive equal the reference's (fixture written
    by the reference code compiled from its sources)."""
    from helpers import assert_bits_equal
    for name, (v, t, m), d in _refpin_scenes():
        sc = orc.Scene(v, t, m)
        b, o, order, _ = sc.export()
        assert_bits_equal(b, d[f"{name}_bounds"], f"{name} bounds")
        assert_bits_equal(o, d[f"{name}_off"], f"{name} offsets")
        assert_bits_equal(order, d[f"{name}_order"], f"{name} order")
        for k, (md, eps, cull) in enumerate(d["settings"]):
            h = sc.trace(d[f"{name}_rays"], max_dist=float(md), eps=float(eps), cullback=bool(cull))
            for key in ("t", "tri", "w", "u", "v"):
                assert_bits_equal(h[key], d[f"{name}_s{k}_{key}"], f"{name} setting {k} {key}")


def test_refpin_fixture_library_builder(gb):
    """The library's threaded BVH builder equals the reference's CreateBVH +
    InitialCompactBVH on the fixture scenes."""
    from helpers import assert_bits_equal
    for name, (v, t, m), d in _refpin_scenes():
        b, o, order = gb.RTScene(v, t, m).build_bvh().bvh_export()
        assert_bits_equal(b, d[f"{name}_bounds"], f"{name} bounds")
        assert_bits_equal(o, d[f"{name}_off"], f"{name} offsets")
        assert_bits_equal(order, d[f"{name}_order"], f"{name} order")


@pytest.mark.gpu
def test_refpin_fixture_gpu(gbdev):
    """The GPU walk (gbpt_trace_rays) returns the reference TracePrimitive's hits
    to the bit: closest hit, back-face culling and the shadow setting."""
    from helpers import assert_bits_equal
    for name, (v, t, m), d in _refpin_scenes():
        s = gbdev.RTScene(v, t, m).build_bvh()
        for k, (md, eps, cull) in enumerate(d["settings"]):
            h = s.trace_rays(d[f"{name}_rays"], max_dist=float(md), eps=float(eps), cullback=bool(cull))
            hit = d[f"{name}_s{k}_tri"] >= 0
            assert_bits_equal(h["tri"], d[f"{name}_s{k}_tri"], f"{name} setting {k} tri")
            for key in ("t", "w", "u", "v"):
                assert_bits_equal(h[key][hit], d[f"{name}_s{k}_{key}"][hit], f"{name} setting {k} {key}")
