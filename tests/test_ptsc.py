"""Unidirectional streaming path tracer "PTSC" (src/cudaRTPTStream.cu) on the
BDPT wavefront: the oracle's semantics on the CPU, GPU parity on the
reference's Cornell OBJ with the glass sphere of its cornellwtranball preset
(refraction and total internal reflection) and on the Cornell box."""
import os

import numpy as np
import pytest

from cudapt_gb300 import layouts
from helpers import assert_bits_equal

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PT = layouts.MODE_PT_SC


def _glass():
    g = np.load(os.path.join(GOLD, "obj_cornell_glass.npz"))
    c = g["cam"]
    cam = dict(pos=tuple(c[0:3]), dir=tuple(c[3:6]), up=tuple(c[6:9]), fov=float(c[9]))
    return (g["vertices"], g["triangles"], g["materials"]), cam


def test_oracle_pt_paths(orc):
    (v, t, m), cam = _glass()
    W, H = 40, 30
    p = layouts.default_params()
    r = orc.Renderer(W, H, PT, p, threads=4)
    sc = orc.Scene(v, t, m)
    r.render(sc, cam, 1)
    st = r.stats()
    assert st["paths"] == W * H and st["rays"] == st["ext_rays"]  # no connections
    assert len(r.light_cache()) == 0 or r.light_cache().shape[0] == 0
    img = r.get(0)
    assert np.all(np.isfinite(img)) and img.min() >= 0.0 and img.max() > 0.0
    first = img.copy()
    r.render(sc, cam, 1)
    # frame weights 1/(f+1): the second frame moves every pixel towards its new sample
    assert r.frame == 1 and not np.array_equal(first, r.get(0))
    assert np.all(r.sample_counts()[0] == 2)


def test_oracle_pt_depth_cap(orc):
    (v, t, m), cam = _glass()
    r1 = orc.Renderer(32, 24, PT, layouts.default_params(pt_depth_max=1), threads=4)
    r1.render(orc.Scene(v, t, m), cam, 1)
    assert r1.stats()["ext_rays"] == 32 * 24  # depth cap 1: the camera ray only


def _both(gb, orc, scene, W, H, frames, **kw):
    (v, t, m), cam = scene
    p = gb.default_params(**kw)
    s = gb.RTScene(v, t, m).build_bvh()
    r = gb.RTRenderer(W, H, PT, p)
    r.set_counting(True)
    for _ in range(frames):
        img = r.render(s, cam).copy()
    ref = orc.Renderer(W, H, PT, p)
    ref.render(orc.Scene(v, t, m), cam, frames)
    return r, ref, img, ref.get(0)


@pytest.mark.gpu
def test_gpu_pt_glass_bitexact(gbdev, orc):
    r, ref, img, want = _both(gbdev, orc, _glass(), 64, 48, 5)
    assert_bits_equal(img, want, "image")
    assert_bits_equal(r.read_buffer(6), ref.sample_counts()[0], "sampleN")
    st, rs = r.last_stats, ref.stats()
    assert st["shadow_rays"] == 0 and st["light_vertices"] == 0
    assert int(st["rays"]) == rs["ext_rays"] and int(st["nodes"]) == rs["ext_nodes"]


@pytest.mark.gpu
def test_gpu_pt_cornell_matches(gbdev, orc):
    from helpers import assert_bits_equal, scene_arrays
    r, ref, img, want = _both(gbdev, orc, scene_arrays("cornell"), 64, 64, 4)
    assert_bits_equal(img, want, "image")
    assert np.array_equal(r.read_buffer(6), np.full(64 * 64, 4, np.uint32))
