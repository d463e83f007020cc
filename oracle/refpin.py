"""The reference's own BVH builder and traversal, built from its sources --
TEST INFRASTRUCTURE ONLY.

``oracle/refpin/Makefile`` compiles ``src/bvhhelper.cpp`` and
``src/cudaRTCommon.cu`` of the CudaPT checkout, unmodified, with the
stand-ins of ``oracle/refpin/prelude.h`` (a g++-compilable Vec3 for the MSVC
one, serial TBB loops, the removed texture references as array views, the
device branch of cudahelper.h with IEEE intrinsics) into
``oracle/_ref/libcudapt_ref.so``.  Tests compare the oracle's restatement
against it, and tests/golden/make_refpin_golden.py writes fixtures from it
that pin the GPU kernels where the checkout is absent.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libcudapt_ref.so")
_lib = None


def build():
    """Runs the recipe; it builds nothing when the reference checkout is absent."""
    subprocess.run(["make", "-s", "-C", os.path.join(_HERE, "refpin")], check=True)
    return LIB_PATH if os.path.exists(LIB_PATH) else None


def available():
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(LIB_PATH)
        vp, u32, i32, f32, u64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int32, ctypes.c_float, ctypes.c_uint64
        L.refpin_scene_create.restype = vp
        L.refpin_scene_create.argtypes = [vp, u32, vp, u32, vp]
        L.refpin_scene_destroy.argtypes = [vp]
        L.refpin_scene_export.argtypes = [vp, vp, vp, vp, vp]
        L.refpin_trace.argtypes = [vp, vp, u32, f32, f32, i32, vp, vp, vp, vp, vp, vp]
        L.refpin_intersect_aabb.argtypes = [vp, u32, vp]
        L.refpin_intersect_tri.argtypes = [vp, u32, f32, i32, vp]
        L.refpin_texture_set.argtypes = [u64, vp, i32, i32]
        L.refpin_material_colors.argtypes = [vp, vp, u32, vp, u32, vp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data if a is not None else None


class RefScene:
    """RTScene::AddModel's BVH set-up over (vertices, triangles): the
    reference's CreateBVH, triangle reorder and InitialCompactBVH."""

    def __init__(self, verts, tris):
        pos = np.ascontiguousarray(verts["pos"], np.float32).reshape(-1, 3)
        idx = np.ascontiguousarray(np.stack([tris["v0"], tris["v1"], tris["v2"]], 1), np.uint32)
        n = ctypes.c_uint32(0)
        self.h = lib().refpin_scene_create(_p(pos), len(pos), _p(idx), len(idx), ctypes.byref(n))
        if not self.h:
            raise RuntimeError("reference BVH build failed")
        self.node_count = n.value
        self.ntri = len(idx)

    def __del__(self):
        if getattr(self, "h", None):
            lib().refpin_scene_destroy(self.h)
            self.h = None

    def export(self):
        b = np.zeros((self.node_count, 6), np.float32)
        o = np.zeros((self.node_count, 2), np.uint32)
        order = np.zeros(self.ntri, np.uint32)
        isect = np.zeros((self.ntri, 9), np.float32)
        lib().refpin_scene_export(self.h, _p(b), _p(o), _p(order), _p(isect))
        return b, o, order, isect

    def trace(self, rays, max_dist=1e20, eps=1e-9, cullback=False):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        n = len(rays)
        hit = np.zeros(n, np.uint8)
        t = np.zeros(n, np.float32)
        tri = np.zeros(n, np.int32)
        w, u, v = (np.zeros(n, np.float32) for _ in range(3))
        lib().refpin_trace(self.h, _p(rays), n, max_dist, eps, int(cullback), _p(hit), _p(t), _p(tri), _p(w), _p(u),
                           _p(v))
        return dict(t=t, tri=tri, w=w, u=u, v=v)


def intersect_aabb(cases):
    """CURay::IntersectAABB over (n, 12) cases: origin, direction, min, max."""
    cases = np.ascontiguousarray(cases, np.float32).reshape(-1, 12)
    out = np.zeros(len(cases), np.float32)
    lib().refpin_intersect_aabb(_p(cases), len(cases), _p(out))
    return out


def intersect_tri(cases, eps=1e-9, cullback=True):
    """CURay::IntersectTri over (n, 15) cases: origin, direction, p0, e0, e1;
    returns (n, 4) t, w, u, v."""
    cases = np.ascontiguousarray(cases, np.float32).reshape(-1, 15)
    out = np.zeros((len(cases), 4), np.float32)
    lib().refpin_intersect_tri(_p(cases), len(cases), eps, int(cullback), _p(out))
    return out


def set_texture(tex_id, rgba):
    """Registers an (H, W, 4) float texture for the tex2D stand-in under tex_id >= 1."""
    rgba = np.ascontiguousarray(rgba, np.float32)
    lib().refpin_texture_set(tex_id, _p(rgba), rgba.shape[1], rgba.shape[0])


def material_colors(mat, uv, tex_ids):
    """GetMaterialColors of one MATERIAL record at (n, 2) uv: (n, 8) = diffuse,
    emissive, transparency, 0."""
    m = np.ascontiguousarray(np.asarray(mat).reshape(()))
    uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
    ids = np.ascontiguousarray(tex_ids, np.uint64)
    out = np.zeros((len(uv), 8), np.float32)
    lib().refpin_material_colors(m.ctypes.data, _p(uv), len(uv), _p(ids) if len(ids) else None, len(ids), _p(out))
    return out
