"""Regenerate the golden fixtures of tests/golden/ (run in the build container).

Inputs:
  * the reference's own Cornell asset ``asset/model/cornell_box_with_sphere.obj``
    (416 faces -> 792 triangles), read from the CudaPT checkout whose root
    is the required command-line argument, positions only;
  * the 36-triangle procedural Cornell box of cudapt_gb300.scenes.

Outputs (all produced by the CPU oracle, FP32 float contract):
  obj_cornell.npz   mesh, BVH (bounds/offsets/order) and 1024 traced rays
  cornell_frames.npz 3 progressive frames of a 24x24 plain-BDPT render and
                     the light-vertex cache of frame 0
  empty_children.npz a 38-triangle scene whose tree has empty children
  obj_cornell_glass.npz the OBJ with its MTL materials, the sphere made glass
                     as the reference's cornellwtranball preset does, and that
                     preset's camera (a scene with refraction and total
                     internal reflection)
The Philox4x32-10 known-answer vectors are the published Random123 ones and
live in the test itself.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from cudapt_gb300 import layouts, objio, scenes  # noqa: E402


def main(ref_root):
    obj = os.path.join(ref_root, "asset", "model", "cornell_box_with_sphere.obj")
    v, t, m = objio.load_obj(obj, with_materials=False)
    sc = oracle.Scene(v, t, m)
    b, o, order, isect = sc.export()
    rng = np.random.Generator(np.random.PCG64(2024))
    p = v["pos"]
    lo, hi = p.min(0), p.max(0)
    orig = (lo + (hi - lo) * rng.random((1024, 3))).astype(np.float32)
    d = rng.normal(size=(1024, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([orig, d.astype(np.float32)], 1).astype(np.float32)
    hits = sc.trace(rays, eps=1e-4)
    np.savez_compressed(os.path.join(HERE, "obj_cornell.npz"), vertices=v, triangles=t, materials=m,
                        bounds=b, off=o, order=order, rays=rays, **{"hit_" + k: hits[k] for k in hits})

    (v2, t2, m2), cam = scenes.cornell()
    sc2 = oracle.Scene(v2, t2, m2)
    params = layouts.default_params(eye_depth_max=8, light_depth_max=8)
    r = oracle.Renderer(24, 24, 0, params, threads=1)
    frames = []
    cache = None
    for f in range(3):
        r.render(sc2, cam, 1)
        frames.append(r.get(0))
        if f == 0:
            cache = r.light_cache()
    np.savez_compressed(os.path.join(HERE, "cornell_frames.npz"), vertices=v2, triangles=t2, materials=m2,
                        cam=oracle.cam_array(cam), params=params, frames=np.array(frames), cache=cache,
                        sampleN=r.sample_counts()[0])
    # the same OBJ with its MTL materials and the preset's glass sphere
    # (asset/preset/cornellwtranball.NPRTENV: transparency 1, roughness 0) and camera
    from cudapt_gb300 import preset
    v3, t3, m3 = objio.load_obj(obj, with_materials=True)
    pre = preset.load(os.path.join(HERE, "cornellwtranball.NPRTENV"))
    glass = int(np.argmax(np.bincount(t3["mat"])))  # the sphere holds most triangles
    m3[glass]["transparency"] = 1.0
    m3[glass]["roughness"] = 0.0
    cam3 = pre["camera"]
    np.savez_compressed(os.path.join(HERE, "obj_cornell_glass.npz"), vertices=v3, triangles=t3, materials=m3,
                        cam=oracle.cam_array(cam3))
    # a small scene whose binned-SAH tree has empty children (kept as (start, 0)
    # records that the reference's walk treats as inner nodes): the first
    # scene of a seeded search of clustered triangles where the oracle's
    # builder reports empty children
    rng = np.random.Generator(np.random.PCG64(0))
    for _ in range(5000):
        n = int(rng.integers(3, 40))
        cen = rng.normal(size=(n, 3)) * rng.choice([1e-3, 1.0, 100.0], size=(n, 1))
        if rng.random() < 0.5:
            cen[: n // 2] = cen[0]
        tri = cen[:, None, :] + rng.normal(size=(n, 3, 3)) * rng.choice([1e-4, 0.5, 20], size=(n, 1, 1))
        v4 = np.zeros(n * 3, layouts.VERTEX)
        v4["pos"] = tri.reshape(-1, 3).astype(np.float32)
        t4 = np.zeros(n, layouts.TRIANGLE)
        t4["v0"] = np.arange(n) * 3
        t4["v1"] = t4["v0"] + 1
        t4["v2"] = t4["v0"] + 2
        m4 = np.zeros(1, layouts.MATERIAL)
        m4[0] = layouts.material()  # untextured (texture ids -1)
        if oracle.Scene(v4, t4, m4).empty_children > 0:
            np.savez_compressed(os.path.join(HERE, "empty_children.npz"), vertices=v4, triangles=t4, materials=m4)
            break
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_golden.py <CudaPT checkout root>")
    main(sys.argv[1])
