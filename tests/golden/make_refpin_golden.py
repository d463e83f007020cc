"""Write tests/golden/refpin_traces.npz from the reference's own code (run in
the build container, where the CudaPT checkout is).

    python tests/golden/make_refpin_golden.py <CudaPT checkout root>

The pin library (oracle/refpin: src/bvhhelper.cpp and src/cudaRTCommon.cu
compiled from the checkout with the stand-ins of oracle/refpin/prelude.h)
builds each scene's BVH as RTScene::AddModel does and traces rays with
TracePrimitive.  The fixture keeps, per scene: positions and triangle
indices (so no generator runs again elsewhere), the reference's node
bounds, child/leaf words and triangle order, and for 2048 rays the hit
(t, reordered triangle id, w, u, v; t = -1 and id -1 on a miss) under
three settings: closest hit (epsilon 1e-9), closest hit with back-face
culling, and a shadow-style query (epsilon 1e-4, distance cap 7.5).
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from cudapt_gb300 import layouts, objio, scenes  # noqa: E402
from helpers import camera_rays, random_rays  # noqa: E402

SETTINGS = ((1e20, 1e-9, 0), (1e20, 1e-9, 1), (7.5, 1e-4, 0))


def _soup(n, seed, spread=10.0, size=0.5):
    rng = np.random.Generator(np.random.PCG64(seed))
    mb = scenes.MeshBuilder()
    mat = mb.add_material(layouts.material((0.5, 0.5, 0.5)))
    c = rng.random((n, 1, 3)) * spread
    mb.add_tris(c + (rng.random((n, 3, 3)) - 0.5) * size, mat)
    return mb.build()


def main(ref_root):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "refpin"), f"REF={ref_root}", "-B"], check=True)
    from oracle import refpin
    if not refpin.available():
        raise SystemExit("the pin library was not built")
    (vc, tc, _), cam_c = scenes.cornell()
    vo, to, _ = objio.load_obj(os.path.join(ref_root, "asset", "model", "cornell_box_with_sphere.obj"),
                               with_materials=False)
    (vi, ti, _), cam_i = scenes.interior(spheres=10, level=2)
    ec = np.load(os.path.join(HERE, "empty_children.npz"))
    vs, ts, _ = _soup(1000, 12)
    todo = {"cornell": (vc, tc, cam_c), "obj_cornell": (vo, to, None), "interior10": (vi, ti, cam_i),
            "empty_children": (ec["vertices"], ec["triangles"], None), "soup1000": (vs, ts, None)}
    out = {}
    for name, (v, t, cam) in todo.items():
        rs = refpin.RefScene(v, t)
        b, o, order, _ = rs.export()
        rays = random_rays(v, 1536 if cam is not None else 2048, 101)
        if cam is not None:
            rays = np.concatenate([rays, camera_rays(cam, 32, 16, 102)])
        out[f"{name}_pos"] = np.ascontiguousarray(v["pos"], np.float32)
        out[f"{name}_idx"] = np.stack([t["v0"], t["v1"], t["v2"]], 1).astype(np.uint32)
        out[f"{name}_bounds"], out[f"{name}_off"], out[f"{name}_order"] = b, o, order
        out[f"{name}_rays"] = rays
        for k, (md, eps, cull) in enumerate(SETTINGS):
            h = rs.trace(rays, max_dist=md, eps=eps, cullback=bool(cull))
            for key in ("t", "tri", "w", "u", "v"):
                out[f"{name}_s{k}_{key}"] = h[key]
    out["settings"] = np.array(SETTINGS, np.float64)
    out["names"] = np.array(sorted(todo))
    np.savez_compressed(os.path.join(HERE, "refpin_traces.npz"), **out)
    print("wrote refpin_traces.npz", os.path.getsize(os.path.join(HERE, "refpin_traces.npz")), "bytes")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_refpin_golden.py <CudaPT checkout root>")
    main(sys.argv[1])
