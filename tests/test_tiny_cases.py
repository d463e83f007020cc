"""Edge cases of whole frames against the oracle: images of 1x1, 4x4 and 3x5
pixels (ragged, smaller than the filter window and than a warp) and a scene
of two triangles (one lit floor triangle, one emissive triangle above it),
in every renderer mode."""
import numpy as np
import pytest

from cudapt_gb300 import layouts, scenes
from helpers import assert_bits_equal

pytestmark = pytest.mark.gpu


def _two_triangles():
    mb = scenes.MeshBuilder()
    floor = mb.add_material(layouts.material((0.7, 0.6, 0.5), specular=0.5, roughness=0.4))
    light = mb.add_material(layouts.material((0.8, 0.8, 0.8), emissive=(9.0, 9.0, 9.0)))
    mb.add_tris([[[-2, 0, -2], [-2, 0, 2], [2, 0, 0]]], floor)
    mb.add_tris([[[-0.5, 1.5, -0.5], [0.5, 1.5, -0.5], [0.0, 1.5, 0.5]]], light)
    cam = {"pos": [0.0, 0.8, 3.0], "dir": [0.0, -0.2, -1.0], "up": [0.0, 1.0, 0.0], "fov": 0.9}
    return mb.build(), cam


@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("W,H", [(1, 1), (4, 4), (3, 5)])
def test_tiny_frames_match_oracle(gbdev, orc, mode, W, H):
    (v, t, m), cam = _two_triangles()
    p = gbdev.default_params(eye_depth_max=5, light_depth_max=5, pt_depth_max=5, warmup_frames=2, filter_radius=5)
    s = gbdev.RTScene(v, t, m).build_bvh()
    r = gbdev.RTRenderer(W, H, mode, p)
    for _ in range(5):
        r.render(s, cam)
    img = r.read_buffer(0)  # the running means (the filter-only mode's image is its filtered view)
    ref = orc.Renderer(W, H, mode, p)
    ref.render(orc.Scene(v, t, m), cam, 5)
    want = ref.get(0)
    assert np.isfinite(img).all()
    assert_bits_equal(img, want, "image")
    assert_bits_equal(r.read_buffer(6), ref.sample_counts()[0], "sampleN")
