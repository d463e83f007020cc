"""CPU oracle of the GB300 BDPT library -- TEST INFRASTRUCTURE ONLY.

A C++ restatement of CudaPT's BDPT hot path (BVH build, traversal, the
streaming BDPT estimator, the adaptive allocator and the bilateral filter),
compiled from the sources in this folder by ``build()`` and loaded with
ctypes.  Only tests/, ``__graft_entry__.smoke()`` and the CPU baseline of
bench.py use it, always as the checker; the shipped library never loads it.

Parity status: pinned.  The reference's own BVH builder and traversal
(src/bvhhelper.cpp, src/cudaRTCommon.cu) compile here from the checkout with
the stand-ins of refpin/prelude.h (oracle/refpin, loaded by
``oracle.refpin``); the oracle's BVH, intersection routines and
TracePrimitive equal them to the bit (tests/test_refpin.py), and
tests/golden/refpin_traces.npz carries their output to machines without the
checkout.  The estimator above the traversal (shading, connections, the
adaptive allocator, the filter) follows the reference line by line; its
transcendentals are the project's own, and the reference's RNG (curand
XORWOW) is replaced by Philox4x32-10, pinned by the published Random123
known-answer vectors.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lock = threading.Lock()
_lib = None


def build(force=False):
    """Compile liboracle.so with the Makefile in this folder."""
    args = ["make", "-s", "-C", _HERE]
    if force:
        args.insert(1, "-B")
    subprocess.run(args, check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(_LIB_PATH):
                build()
            L = ctypes.CDLL(_LIB_PATH)
            vp, u32, i32, f32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int32, ctypes.c_float
            L.orc_scene_create.restype = vp
            L.orc_scene_create.argtypes = [vp, u32, vp, u32, vp, u32, vp]
            L.orc_scene_destroy.argtypes = [vp]
            for n in ("orc_scene_node_count", "orc_scene_empty_children", "orc_scene_light_count"):
                getattr(L, n).restype = u32
                getattr(L, n).argtypes = [vp]
            L.orc_scene_export.argtypes = [vp, vp, vp, vp, vp]
            L.orc_update_materials.argtypes = [vp, vp, u32]
            L.orc_trace.argtypes = [vp, vp, u32, f32, f32, i32, vp, vp, vp, vp, vp, vp, vp]
            L.orc_intersect_aabb.argtypes = [vp, u32, vp]
            L.orc_scene_set_textures.argtypes = [vp, u32, vp, vp, vp]
            L.orc_texture_sample.argtypes = [vp, u32, u32, vp, u32, vp]
            L.orc_material_colors.argtypes = [vp, vp, u32, u32, vp, vp, vp, vp]
            L.orc_intersect_tri.argtypes = [vp, u32, f32, i32, vp]
            L.orc_default_params.argtypes = [vp]
            L.orc_renderer_create.restype = vp
            L.orc_renderer_create.argtypes = [u32, u32, i32, vp, u32]
            L.orc_renderer_destroy.argtypes = [vp]
            L.orc_renderer_set_params.argtypes = [vp, vp]
            L.orc_renderer_set_window.argtypes = [vp, u32, u32, u32, u32]
            L.orc_render.argtypes = [vp, vp, vp, u32]
            L.orc_renderer_get.argtypes = [vp, i32, vp]
            L.orc_renderer_counts.argtypes = [vp, vp, vp]
            L.orc_renderer_set_debug.argtypes = [vp, u32]
            L.orc_renderer_frame.restype = u32
            L.orc_renderer_frame.argtypes = [vp]
            L.orc_renderer_stats.argtypes = [vp, vp]
            L.orc_renderer_ext_stats.argtypes = [vp, vp]
            L.orc_renderer_light_cache.restype = u32
            L.orc_renderer_light_cache.argtypes = [vp, vp]
            L.orc_render_fp64.argtypes = [vp, vp, u32, u32, vp, u32, u32, vp]
            L.orc_gaussian.argtypes = [f32, u32, vp]
            L.orc_bilateral.argtypes = [vp, vp, vp, vp, u32, u32, f32, f32, f32, f32, u32, vp, vp]
            L.orc_philox.argtypes = [vp, u32, u32, vp]
            L.orc_fmath.argtypes = [i32, vp, u32, vp]
            _lib = L
    return _lib


def _p(a):
    return a.ctypes.data if a is not None else None


def cam_array(cam):
    return np.array(list(cam["pos"]) + list(cam["dir"]) + list(cam["up"]) + [cam["fov"]], np.float32)


class Scene:
    """Oracle scene: BVH built by the restated builder, triangles reordered."""

    def __init__(self, verts, tris, mats):
        self.verts, self.tris, self.mats = verts, tris, mats
        t = ctypes.c_double(0.0)
        self.h = lib().orc_scene_create(_p(verts), len(verts), _p(tris), len(tris), _p(mats), len(mats),
                                        ctypes.addressof(t))
        if not self.h:
            raise RuntimeError("oracle BVH build failed")
        self.build_seconds = t.value

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_scene_destroy(self.h)
            self.h = None

    @property
    def node_count(self):
        return lib().orc_scene_node_count(self.h)

    @property
    def empty_children(self):
        return lib().orc_scene_empty_children(self.h)

    @property
    def light_count(self):
        return lib().orc_scene_light_count(self.h)

    def export(self):
        n = self.node_count
        b = np.zeros((n, 6), np.float32)
        o = np.zeros((n, 2), np.uint32)
        order = np.zeros(len(self.tris), np.uint32)
        isect = np.zeros((len(self.tris), 9), np.float32)
        lib().orc_scene_export(self.h, _p(b), _p(o), _p(order), _p(isect))
        return b, o, order, isect

    def update_materials(self, mats):
        self.mats = mats
        lib().orc_update_materials(self.h, _p(mats), len(mats))

    def set_textures(self, textures):
        """RTScene::m_pTextures: (H, W, 4) float RGBA arrays, row 0 first."""
        arrs = [np.ascontiguousarray(t, np.float32) for t in textures]
        w = np.array([a.shape[1] for a in arrs], np.uint32)
        h = np.array([a.shape[0] for a in arrs], np.uint32)
        flat = np.concatenate([a.reshape(-1) for a in arrs]) if arrs else np.zeros(1, np.float32)
        lib().orc_scene_set_textures(self.h, len(arrs), _p(w), _p(h), _p(flat))
        self.textures = arrs

    def trace(self, rays, max_dist=1e20, eps=1e-9, cullback=False):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        n = len(rays)
        t = np.zeros(n, np.float32)
        tid = np.zeros(n, np.int32)
        w, u, v = (np.zeros(n, np.float32) for _ in range(3))
        nodes = np.zeros(n, np.uint32)
        trs = np.zeros(n, np.uint32)
        lib().orc_trace(self.h, _p(rays), n, max_dist, eps, int(cullback), _p(t), _p(tid), _p(w), _p(u), _p(v),
                        _p(nodes), _p(trs))
        return dict(t=t, tri=tid, w=w, u=u, v=v, nodes=nodes, tris=trs)


class Renderer:
    """Oracle renderer: one call of render() adds `frames` progressive passes."""

    def __init__(self, width, height, mode, params, threads=None):
        from cudapt_gb300.layouts import as_params
        self.W, self.H = width, height
        self.params = as_params(params)
        self.h = lib().orc_renderer_create(width, height, mode, _p(self.params), threads or os.cpu_count())

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_renderer_destroy(self.h)
            self.h = None

    def set_window(self, x0, y0, full_w, full_h):
        """Render only the W x H window at (x0, y0) of a full_w x full_h image."""
        lib().orc_renderer_set_window(self.h, x0, y0, full_w, full_h)

    def render(self, scene, cam, frames=1):
        c = cam_array(cam)
        lib().orc_render(self.h, scene.h, _p(c), frames)

    def set_debug(self, mode):
        """Debug view of the filter-only mode (0..7)."""
        lib().orc_renderer_set_debug(self.h, mode)

    def get(self, which=0):
        """0 result, 1 position, 2 normal, 3 diffuse, 4 filtered, 5 error; filter-only
        mode: 8 direct, 9 first-hit emissive, 10 mean 1 - potential, 11 the debug view."""
        n = self.W * self.H * (1 if which in (5, 10) else 3)
        out = np.zeros(n, np.float32)
        lib().orc_renderer_get(self.h, which, _p(out))
        return out

    def sample_counts(self):
        sn = np.zeros(self.W * self.H, np.uint32)
        cn = np.zeros(self.W * self.H, np.uint32)
        lib().orc_renderer_counts(self.h, _p(sn), _p(cn))
        return sn, cn

    @property
    def frame(self):
        return lib().orc_renderer_frame(self.h)

    def stats(self):
        s = np.zeros(4, np.uint64)
        lib().orc_renderer_stats(self.h, _p(s))
        e = np.zeros(3, np.uint64)
        lib().orc_renderer_ext_stats(self.h, _p(e))
        return dict(paths=int(s[0]), rays=int(s[1]), nodes=int(s[2]), tris=int(s[3]), ext_rays=int(e[0]),
                    ext_nodes=int(e[1]), ext_tris=int(e[2]))

    def light_cache(self):
        n = lib().orc_renderer_light_cache(self.h, None)
        out = np.zeros((max(n, 1), 21), np.float32)
        lib().orc_renderer_light_cache(self.h, _p(out))
        return out[:n]


def intersect_aabb(cases):
    """IntersectAABB over (n, 12) cases: origin, direction, min, max."""
    cases = np.ascontiguousarray(cases, np.float32).reshape(-1, 12)
    out = np.zeros(len(cases), np.float32)
    lib().orc_intersect_aabb(_p(cases), len(cases), _p(out))
    return out


def intersect_tri(cases, eps=1e-9, cullback=True):
    """IntersectTri over (n, 15) cases: origin, direction, p0, e0, e1; (n, 4) t, w, u, v."""
    cases = np.ascontiguousarray(cases, np.float32).reshape(-1, 15)
    out = np.zeros((len(cases), 4), np.float32)
    lib().orc_intersect_tri(_p(cases), len(cases), eps, int(cullback), _p(out))
    return out


def texture_sample(rgba, uv):
    """The linear-filtered, wrapped fetch of an (H, W, 4) texture at (n, 2) uv (texture_ref.h)."""
    rgba = np.ascontiguousarray(rgba, np.float32)
    uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
    out = np.zeros((len(uv), 4), np.float32)
    lib().orc_texture_sample(_p(rgba), rgba.shape[1], rgba.shape[0], _p(uv), len(uv), _p(out))
    return out


def material_colors(mat, uv, textures):
    """GetMaterialColors' colours of one MATERIAL record at (n, 2) uv with
    (H, W, 4) textures: (n, 8) = diffuse, emissive, transparency, 0."""
    arrs = [np.ascontiguousarray(t, np.float32) for t in textures]
    w = np.array([a.shape[1] for a in arrs] or [0], np.uint32)
    h = np.array([a.shape[0] for a in arrs] or [0], np.uint32)
    flat = np.concatenate([a.reshape(-1) for a in arrs]) if arrs else np.zeros(1, np.float32)
    m = np.ascontiguousarray(np.asarray(mat).reshape(()))
    uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
    out = np.zeros((len(uv), 8), np.float32)
    lib().orc_material_colors(m.ctypes.data, _p(uv), len(uv), len(arrs), _p(w), _p(h), _p(flat), _p(out))
    return out


def render_fp64(scene, params, width, height, cam, frames, threads=None):
    from cudapt_gb300.layouts import as_params
    out = np.zeros(width * height * 3, np.float64)
    c = cam_array(cam)
    p = as_params(params)
    lib().orc_render_fp64(scene.h, _p(p), width, height, _p(c), frames, threads or os.cpu_count(), _p(out))
    return out


def gaussian(delta, radius):
    g = np.zeros(64, np.float32)
    lib().orc_gaussian(delta, radius, _p(g))
    return g


def bilateral(color, pos, norm, emit, W, H, ceud, peud, neud, eeud, radius, g):
    out = np.zeros(W * H * 3, np.float32)
    args = [np.ascontiguousarray(a, np.float32) if a is not None else None for a in (color, pos, norm, emit)]
    lib().orc_bilateral(*[_p(a) for a in args], W, H, ceud, peud, neud, eeud, radius, _p(g), _p(out))
    return out


def philox(ctr, k0, k1):
    c = np.array(ctr, np.uint32)
    out = np.zeros(4, np.uint32)
    lib().orc_philox(_p(c), k0, k1, _p(out))
    return out


def fmath(which, x):
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros_like(x)
    lib().orc_fmath({"sin": 0, "cos": 1, "exp": 2, "sqrt_rd": 3, "pow5": 4}[which], _p(x), len(x), _p(out))
    return out
