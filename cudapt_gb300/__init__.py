"""cudapt_gb300 -- GB300-native streaming bidirectional path tracer.

Host-side mirror of CudaPT's scene/renderer surface (include/raytracer.h:
``RTScene``, ``RTRenderer``) over the C ABI of ``libgbpt.so``
(include/gbpt.h).  All rendering runs in hand-written CUDA kernels for
sm_103a; this module only moves arrays and handles.
"""
import ctypes

import numpy as np

from . import _native, layouts
from ._native import GbptError, Stats, as_c, check, load, ptr
from .layouts import (MATERIAL, MODE_BDPT_SC, MODE_BDPT_SC_ADAP_BILAT, MODE_BDPT_SC_ADAP_BILAT_BINARY,
                      MODE_BDPT_SC_BILAT, MODE_PT_SC, PARAMS, TRIANGLE, VERTEX, default_params, material)

__all__ = [
    "RTScene", "RTRenderer", "GbptError", "default_params", "material", "layouts",
    "MODE_BDPT_SC", "MODE_BDPT_SC_ADAP_BILAT", "MODE_BDPT_SC_ADAP_BILAT_BINARY", "MODE_BDPT_SC_BILAT", "MODE_PT_SC",
    "VERTEX",
    "TRIANGLE", "MATERIAL", "PARAMS",
    "device_available", "camera",
]


def device_available():
    """True when a CUDA device runs the library's kernels."""
    ok = ctypes.c_int32(0)
    st = load().gbpt_device_check(ctypes.addressof(ok))
    return st == 0 and ok.value == 1


def camera(pos, dir, up, fov):
    c = np.array(list(pos) + list(dir) + list(up) + [fov], np.float32)
    return c


class RTScene:
    """Scene arrays in CudaPT's layouts (RTVertex / RTTriangle / RTMaterial).

    ``build_bvh()`` is ``RTScene::AddModel``'s BVH part
    (src/raytracer.cpp:264-281): binned-SAH build, triangle reorder, upload.
    """

    def __init__(self, vertices, triangles, materials):
        L = load()
        self.vertices = as_c(vertices, VERTEX)
        self.triangles = as_c(triangles, TRIANGLE)
        self.materials = as_c(materials, MATERIAL)
        h = ctypes.c_void_p()
        check(L.gbpt_scene_create(ptr(self.vertices), len(self.vertices), ptr(self.triangles), len(self.triangles),
                                  ptr(self.materials), len(self.materials), ctypes.addressof(h)))
        self._h = h
        self.build_seconds = None

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            load().gbpt_scene_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build_bvh(self, max_depth=32, threads=0):
        t = ctypes.c_double(0.0)
        check(load().gbpt_scene_build_bvh(self._h, max_depth, threads, ctypes.addressof(t)))
        self.build_seconds = t.value
        return self

    def update_materials(self, materials):
        self.materials = as_c(materials, MATERIAL)
        check(load().gbpt_scene_update_materials(self._h, ptr(self.materials), len(self.materials)))

    def set_textures(self, textures):
        """RTScene::m_pTextures: a list of (H, W, 4) float RGBA arrays (row 0
        first), indexed by the materials' diffuseTexId / emissiveTexId."""
        arrs = [np.ascontiguousarray(t, np.float32) for t in textures]
        for a in arrs:
            if a.ndim != 3 or a.shape[2] != 4:
                raise ValueError("a texture is an (H, W, 4) float array")
        rec = (_native.Texture * max(len(arrs), 1))()
        for i, a in enumerate(arrs):
            rec[i].rgba = a.ctypes.data
            rec[i].width = a.shape[1]
            rec[i].height = a.shape[0]
        check(load().gbpt_scene_set_textures(self._h, ctypes.addressof(rec), len(arrs)))
        self.textures = arrs  # kept for the caller's inspection; the library holds its own copy
        return self

    def set_traversal(self, mode):
        """BVH walk order: 0 / "reference" (bit-exact with TracePrimitive, the default) or
        1 / "wide" (collapsed 4-ary tree, nearest child first; same closest hits)."""
        m = {"reference": 0, "wide": 1}.get(mode, mode)
        check(load().gbpt_scene_set_traversal(self._h, int(m)))
        return self

    def bvh_info(self):
        n, t, l = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        check(load().gbpt_scene_bvh_info(self._h, ctypes.addressof(n), ctypes.addressof(t), ctypes.addressof(l)))
        return dict(nodes=n.value, tris=t.value, lights=l.value)

    def bvh_export(self):
        info = self.bvh_info()
        b = np.zeros((info["nodes"], 6), np.float32)
        o = np.zeros((info["nodes"], 2), np.uint32)
        order = np.zeros(info["tris"], np.uint32)
        check(load().gbpt_scene_bvh_export(self._h, ptr(b), ptr(o), ptr(order)))
        return b, o, order

    def trace_rays(self, rays, max_dist=1e20, eps=1e-9, cullback=False, counts=False):
        """TracePrimitive on the GPU for (n, 6) rays: closest hit t / tri / w,u,v."""
        rays = as_c(rays, np.float32).reshape(-1, 6)
        n = len(rays)
        t = np.zeros(n, np.float32)
        tri = np.zeros(n, np.int32)
        w, u, v = (np.zeros(n, np.float32) for _ in range(3))
        nodes = np.zeros(n, np.uint32) if counts else None
        tt = np.zeros(n, np.uint32) if counts else None
        check(load().gbpt_trace_rays(self._h, ptr(rays), n, max_dist, eps, int(cullback), ptr(t), ptr(tri), ptr(w),
                                     ptr(u), ptr(v), ptr(nodes), ptr(tt), 0))
        out = dict(t=t, tri=tri, w=w, u=u, v=v)
        if counts:
            out.update(nodes=nodes, tris=tt)
        return out


_PAGE = 4096


def _host_floats(n):
    """A zeroed float32 host array of n values on whole pages of its own,
    page-locked through gbpt_host_register when CUDA allows it (the result
    copy of gbpt_render then runs at link speed).  Returns (array, the
    registered address or None)."""
    nbytes = n * 4
    span = -(-nbytes // _PAGE) * _PAGE
    raw = np.zeros(span + _PAGE, np.uint8)
    off = (-raw.ctypes.data) % _PAGE
    arr = raw[off:off + nbytes].view(np.float32)
    addr = raw.ctypes.data + off
    if load().gbpt_host_register(ctypes.c_void_p(addr), span) != 0:
        return arr, None
    return arr, ctypes.c_void_p(addr)


class RTRenderer:
    """``RTRenderer`` (include/raytracer.h:292-323) for the BDPT modes.

    ``render()`` adds one progressive pass (``RTRenderer::Render``) and
    returns the W*H*3 float image (row 0 at the bottom); the frame counter
    restarts when the camera changes, as in the reference.
    """

    def __init__(self, width, height, mode=MODE_BDPT_SC, params=None):
        L = load()
        self.width, self.height = int(width), int(height)
        p = layouts.as_params(params)
        h = ctypes.c_void_p()
        check(L.gbpt_renderer_create(self.width, self.height, int(mode), ptr(p), ctypes.addressof(h)))
        self._h = h
        self._mode = int(mode)
        self._out, self._pinned = _host_floats(self.width * self.height * 3)
        self.last_stats = None

    # reference-style names
    def Init(self, width, height):  # noqa: N802
        params, mode = self.params, self.mode
        self.close()
        self.__init__(width, height, mode, params)
        return True

    def SetRendererMode(self, mode):  # noqa: N802
        check(load().gbpt_set_mode(self._h, int(mode)))
        self._mode = int(mode)

    def Render(self, camPos, camDir, camUp, fov, scene):  # noqa: N802,N803
        self.render(scene, camera(camPos, camDir, camUp, fov))
        return True

    def GetResult(self):  # noqa: N802
        return self._out

    @property
    def mode(self):
        return self._mode

    @property
    def handle(self):
        return self._h

    def checkpoint(self):
        """The renderer's whole progressive state as bytes (gbpt_renderer_checkpoint)."""
        n = ctypes.c_size_t()
        check(load().gbpt_renderer_checkpoint_size(self._h, ctypes.addressof(n)))
        buf = np.empty(n.value, np.uint8)
        check(load().gbpt_renderer_checkpoint(self._h, ptr(buf), buf.nbytes))
        return buf.tobytes()

    def restore(self, data):
        """Continue from checkpoint() bytes: the next render with the same scene and
        camera gives the frame the interrupted renderer would have given."""
        buf = np.frombuffer(data, np.uint8)
        check(load().gbpt_renderer_restore(self._h, ptr(buf), buf.nbytes))
        self._mode = int(np.frombuffer(data[20:24], np.int32)[0])  # the header's mode word
        return self

    def set_window(self, x0, y0, full_w, full_h):
        """Render the window at (x0, y0) of a full_w x full_h image (rays and random
        numbers of the full image's pixels); (0, 0, width, height) is the whole image."""
        check(load().gbpt_renderer_set_window(self._h, int(x0), int(y0), int(full_w), int(full_h)))
        return self

    def set_graphs(self, on=True):
        """Issue each frame of the plain and PTSC modes as one CUDA graph (same image)."""
        check(load().gbpt_renderer_set_graphs(self._h, 1 if on else 0))
        return self

    def set_mlp(self, mlp=None, collect=False):
        """Learned allocation with `mlp` (cudapt_gb300.mlp.MLP) in the PLL adaptive mode;
        collect=True keeps the feature statistics without changing the allocation."""
        self._mlp = mlp  # keep the network alive while attached
        check(load().gbpt_renderer_set_mlp(self._h, mlp.handle if mlp is not None else None, int(bool(collect))))

    def features(self):
        """(tiles, 24) features of the current statistics (row-major 8x8 tiles)."""
        n = ctypes.c_uint32()
        check(load().gbpt_renderer_features(self._h, None, 0, 0, ctypes.addressof(n)))
        out = np.zeros((n.value, 24), np.float32)
        check(load().gbpt_renderer_features(self._h, ptr(out), n.value, 0, ctypes.addressof(n)))
        return out

    def rmse(self, converged):
        """RMSE of the current image against a converged W*H*3 image (on the GPU)."""
        from .experiment import renderer_rmse
        return renderer_rmse(self, converged)

    @property
    def params(self):
        p = np.zeros((), PARAMS)
        check(load().gbpt_get_params(self._h, ptr(p)))
        return p

    @params.setter
    def params(self, p):
        p = layouts.as_params(p)
        check(load().gbpt_set_params(self._h, ptr(p)))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            load().gbpt_renderer_destroy(self._h)
            self._h = ctypes.c_void_p()
        if getattr(self, "_pinned", None):
            load().gbpt_host_unregister(self._pinned)  # the array stays valid, as pageable memory
            self._pinned = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _cam(self, cam):
        if isinstance(cam, dict):
            cam = camera(cam["pos"], cam["dir"], cam["up"], cam["fov"])
        return as_c(cam, np.float32)

    def render(self, scene, cam, stats=True):
        c = self._cam(cam)
        s = Stats() if stats else None
        check(load().gbpt_render(self._h, scene.handle, ptr(c), ptr(self._out), 0,
                                 ctypes.addressof(s) if s is not None else None))
        self.last_stats = s.as_dict() if s is not None else None
        return self._out

    def render_frames(self, scene, cam, frames, stats=True):
        c = self._cam(cam)
        s = Stats() if stats else None
        check(load().gbpt_render_frames(self._h, scene.handle, ptr(c), int(frames),
                                        ctypes.addressof(s) if s is not None else None))
        self.last_stats = s.as_dict() if s is not None else None
        return self.last_stats

    def read_buffer(self, which):
        """0 result, 1 position, 2 normal, 3 diffuse, 4 filtered, 5 error, 6 sample count;
        filter-only mode: 8 direct light, 9 first-hit emissive, 10 mean of 1 - path potential."""
        np_ = self.width * self.height
        if which in (5, 10):
            out = np.zeros(np_, np.float32)
        elif which == 12:
            out = np.zeros(((self.width + 7) // 8) * ((self.height + 7) // 8) * 8, np.uint32)
        elif which == 6:
            out = np.zeros(np_, np.uint32)
        else:
            out = np.zeros(np_ * 3, np.float32)
        check(load().gbpt_read_buffer(self._h, which, ptr(out), out.nbytes, 0))
        return out

    def light_cache(self, n):
        """First n light vertices in the reference's LightVertex field order (21 floats)."""
        out = np.zeros((max(n, 1), 21), np.float32)
        check(load().gbpt_read_buffer(self._h, 7, ptr(out), out.nbytes, 0))
        return out[:n]

    def reset(self):
        check(load().gbpt_reset(self._h))

    def clean(self):
        check(load().gbpt_clean(self._h))

    def set_counting(self, on):
        check(load().gbpt_set_counting(self._h, int(bool(on))))

    def attr_names(self):
        n = ctypes.c_uint32()
        check(load().gbpt_attr_count(self._h, ctypes.addressof(n)))
        names = []
        buf = ctypes.create_string_buffer(128)
        for i in range(n.value):
            check(load().gbpt_attr_name(self._h, i, buf, 128))
            names.append(buf.value.decode())
        return names

    def attr_get(self, name):
        v = ctypes.c_float()
        check(load().gbpt_attr_get(self._h, name.encode(), ctypes.addressof(v)))
        return v.value

    def attr_set(self, name, value):
        check(load().gbpt_attr_set(self._h, name.encode(), float(value)))
