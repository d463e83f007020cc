"""Wide traversal (gbpt_scene_set_traversal(scene, 1)): the collapsed 4-ary
tree walked nearest child first finds the reference's closest hits -- same
triangle, bit-identical t, u, v -- except where two surfaces lie within the
reference's 1e-4 origin push of each other along the ray: there the answer
depends on the walk order (a triangle is measured from the pushed origin,
its box from the unpushed one, so a walk can cull a box whose triangle is
nearer than the hit it already has), and each walk keeps the surface of the
pair that it reaches first.  The reference order stays the default and the
bit-exact mode."""
import os

import numpy as np
import pytest

from helpers import camera_rays, random_rays, scene_arrays

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _scenes():
    g = np.load(os.path.join(GOLD, "obj_cornell_glass.npz"))
    c = g["cam"]
    glass = ((g["vertices"], g["triangles"], g["materials"]),
             dict(pos=tuple(c[0:3]), dir=tuple(c[3:6]), up=tuple(c[6:9]), fov=float(c[9])))
    return {"cornell": scene_arrays("cornell"), "interior": scene_arrays("interior"),
            "hall_small": scene_arrays("hall_small"), "obj_glass": glass}


@pytest.mark.parametrize("name", ["cornell", "interior", "hall_small", "obj_glass"])
def test_wide_hits_equal_reference(gbdev, orc, name):
    (v, t, m), cam = _scenes()[name]
    rays = np.concatenate([random_rays(v, 150000, 11), camera_rays(cam, 256, 192, 12)])
    ref = orc.Scene(v, t, m).trace(rays, eps=1e-4)
    s = gbdev.RTScene(v, t, m).build_bvh()
    base = s.trace_rays(rays, eps=1e-4)
    s.set_traversal("wide")
    got = s.trace_rays(rays, eps=1e-4)
    for k in ("tri", "t", "u", "v"):  # the default order is the reference's, bit for bit
        assert np.array_equal(np.asarray(base[k]).view(np.uint32), np.asarray(ref[k]).view(np.uint32)), k
    same = got["tri"] == ref["tri"]
    bad = ~same
    # every difference is the other surface of a pair within the origin-push window
    gt, rt = np.asarray(got["t"], np.float64)[bad], np.asarray(ref["t"], np.float64)[bad]
    assert np.all((gt >= 0) & (rt >= 0) & (np.abs(rt - gt) <= 2e-4 * np.maximum(1.0, rt))), name
    assert np.count_nonzero(bad) <= 0.015 * len(rays), (name, np.count_nonzero(bad))
    if name == "interior":  # spheres touch the floor at single points: no coincident surfaces
        assert np.count_nonzero(bad) <= 2, (name, np.count_nonzero(bad))
    for k in ("t", "u", "v"):
        assert np.array_equal(np.asarray(got[k])[same].view(np.uint32), np.asarray(ref[k])[same].view(np.uint32)), k


def test_wide_frames_match_oracle(gbdev, orc):
    for name, W, H, depth in (("cornell", 64, 64, 8), ("interior", 96, 72, 10)):
        (v, t, m), cam = scene_arrays(name)
        p = gbdev.default_params(eye_depth_max=depth, light_depth_max=depth)
        s = gbdev.RTScene(v, t, m).build_bvh().set_traversal("wide")
        r = gbdev.RTRenderer(W, H, 0, p)
        for _ in range(4):
            img = r.render(s, cam).copy()
        ref = orc.Renderer(W, H, 0, p)
        ref.render(orc.Scene(v, t, m), cam, 4)
        want = ref.get(0)
        same = np.mean(img.view(np.uint32) == want.view(np.uint32))
        assert same >= 0.995, (name, same)
        assert abs(img.mean() - want.mean()) <= 1e-3 * want.mean()
