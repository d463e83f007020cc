"""Deterministic procedural scenes standing in for CudaPT's public scenes.

The reference renders Cornell/Sponza/Sibenik/Conference OBJs through Assimp
(src/raytracer.cpp:238-282); those meshes are not available, so these
generators build synthetic scenes with the shapes, sizes and material
distributions of the benchmark workloads:

* ``cornell()``  -- 10-triangle unit room, two boxes (24 triangles), 2-triangle light: 36 triangles.
* ``interior()`` -- 20x10x30 room, 180 jittered icospheres on the floor, one 2x2 light.
* ``hall()``     -- 40x8x40 hall, 12x12 cylindrical pillars, 1200 displaced boxes, 4 lights.

Every triangle carries its own three vertices with the face normal (flat
shading), so the interpolated normal equals the face normal.  Randomness
comes from numpy's PCG64 ``random()``, whose doubles are platform
independent; Gaussian jitter uses the Irwin-Hall sum of twelve uniforms.
"""
import math

import numpy as np

from .layouts import MATERIAL, TRIANGLE, VERTEX, material


class MeshBuilder:
    """Accumulates flat-shaded triangles and materials in reference layouts."""

    def __init__(self):
        self._pos = []      # (n,3,3) float64 corner positions
        self._mat = []      # material id per triangle
        self.materials = []

    def add_material(self, m):
        self.materials.append(m)
        return len(self.materials) - 1

    def add_tris(self, corners, mat_id):
        corners = np.asarray(corners, np.float64).reshape(-1, 3, 3)
        self._pos.append(corners)
        self._mat.append(np.full(len(corners), mat_id, np.uint32))

    def add_quad(self, a, b, c, d, mat_id):
        """Quad a-b-c-d (counter-clockwise seen from the lit side) as two triangles."""
        self.add_tris([[a, b, c], [a, c, d]], mat_id)

    def build(self):
        pos = np.concatenate(self._pos).astype(np.float32)          # (T,3,3)
        mats = np.concatenate(self._mat)
        T = len(pos)
        e0 = (pos[:, 1] - pos[:, 0]).astype(np.float64)
        e1 = (pos[:, 2] - pos[:, 0]).astype(np.float64)
        n = np.cross(e0, e1)
        ln = np.sqrt((n * n).sum(1, keepdims=True))
        ln[ln == 0] = 1.0
        n = (n / ln).astype(np.float32)
        verts = np.zeros(T * 3, VERTEX)
        verts["pos"] = pos.reshape(-1, 3)
        verts["norm"] = np.repeat(n, 3, axis=0)
        tris = np.zeros(T, TRIANGLE)
        idx = np.arange(T * 3, dtype=np.uint32).reshape(T, 3)
        tris["v0"], tris["v1"], tris["v2"] = idx[:, 0], idx[:, 1], idx[:, 2]
        tris["mat"] = mats
        materials = np.array(self.materials, dtype=MATERIAL).reshape(-1)
        return verts, tris, materials


def _box_corners(cx, cz, sx, sy, sz, angle, y0=0.0):
    """8 corners of a y-up box rotated by ``angle`` around its vertical axis."""
    c, s = math.cos(angle), math.sin(angle)
    out = []
    for y in (y0, y0 + sy):
        for (dx, dz) in ((-0.5, -0.5), (0.5, -0.5), (0.5, 0.5), (-0.5, 0.5)):
            lx, lz = dx * sx, dz * sz
            out.append((cx + c * lx + s * lz, y, cz - s * lx + c * lz))
    return np.array(out)


def _box_faces(cn):
    """Six outward quads of a box given its 8 corners (bottom 0-3, top 4-7)."""
    b0, b1, b2, b3, t0, t1, t2, t3 = cn
    return [
        (b0, b3, b2, b1),  # bottom (-y)
        (t0, t1, t2, t3),  # top (+y)
        (b0, b1, t1, t0),  # -z side
        (b1, b2, t2, t1),  # +x side
        (b2, b3, t3, t2),  # +z side
        (b3, b0, t0, t3),  # -x side
    ]


def cornell():
    """Cornell box of the 36-triangle benchmark: unit room open at z=1, white
    0.75 / red / green Lambertian walls (specular 0, so the Fresnel term and
    the reflect probability are zero), a short (0.3) and a tall (0.6) box
    rotated +-17 degrees, a 0.25x0.25 ceiling light of radiance 17."""
    mb = MeshBuilder()
    white = mb.add_material(material((0.75, 0.75, 0.75), specular=0.0, roughness=1.0))
    red = mb.add_material(material((0.63, 0.06, 0.05), specular=0.0, roughness=1.0))
    green = mb.add_material(material((0.14, 0.45, 0.09), specular=0.0, roughness=1.0))
    light = mb.add_material(material((0.75, 0.75, 0.75), emissive=(17.0, 17.0, 17.0), specular=0.0, roughness=1.0))
    P = lambda x, y, z: (x, y, z)  # noqa: E731
    mb.add_quad(P(0, 0, 0), P(0, 0, 1), P(1, 0, 1), P(1, 0, 0), white)    # floor (+y)
    mb.add_quad(P(0, 1, 0), P(1, 1, 0), P(1, 1, 1), P(0, 1, 1), white)    # ceiling (-y)
    mb.add_quad(P(0, 0, 0), P(1, 0, 0), P(1, 1, 0), P(0, 1, 0), white)    # back wall (+z)
    mb.add_quad(P(0, 0, 0), P(0, 1, 0), P(0, 1, 1), P(0, 0, 1), red)      # left wall (+x)
    mb.add_quad(P(1, 0, 0), P(1, 0, 1), P(1, 1, 1), P(1, 1, 0), green)    # right wall (-x)
    ang = math.radians(17.0)
    for (cx, cz, h, a) in ((0.33, 0.62, 0.3, ang), (0.66, 0.33, 0.6, -ang)):
        for q in _box_faces(_box_corners(cx, cz, 0.3, h, 0.3, a)):
            mb.add_quad(*q, white)
    y = 0.999
    mb.add_quad(P(0.375, y, 0.375), P(0.625, y, 0.375), P(0.625, y, 0.625), P(0.375, y, 0.625), light)
    cam = dict(pos=(0.5, 0.5, 2.4), dir=(0.0, 0.0, -1.0), up=(0.0, 1.0, 0.0), fov=math.radians(40.0))
    return mb.build(), cam


def _icosphere(level):
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, np.float64) / math.sqrt(sum(c * c for c in p)) for p in v]
    for _ in range(level):
        cache = {}
        nf = []

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / math.sqrt(float((m * m).sum())))
                cache[key] = len(verts) - 1
            return cache[key]

        for (a, b, c) in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf
    return np.array(verts), np.array(f)


def _gauss(rng, shape):
    return rng.random(shape + (12,)).sum(-1) - 6.0


def _disney(rng):
    """Per-object draw: baseColor U[0.1,0.9]^3, roughness U[0.05,1],
    metallic Bernoulli(0.3), specular 0.5."""
    col = 0.1 + 0.8 * rng.random(3)
    rough = 0.05 + 0.95 * rng.random()
    metal = 1.0 if rng.random() < 0.3 else 0.0
    return material(tuple(col), specular=0.5, metallic=metal, roughness=rough)


def _room(mb, X, Y, Z, mat):
    P = lambda x, y, z: (x, y, z)  # noqa: E731
    mb.add_quad(P(0, 0, 0), P(0, 0, Z), P(X, 0, Z), P(X, 0, 0), mat)    # floor
    mb.add_quad(P(0, Y, 0), P(X, Y, 0), P(X, Y, Z), P(0, Y, Z), mat)    # ceiling
    mb.add_quad(P(0, 0, 0), P(X, 0, 0), P(X, Y, 0), P(0, Y, 0), mat)    # z=0 wall
    mb.add_quad(P(0, 0, Z), P(0, Y, Z), P(X, Y, Z), P(X, 0, Z), mat)    # z=Z wall
    mb.add_quad(P(0, 0, 0), P(0, Y, 0), P(0, Y, Z), P(0, 0, Z), mat)    # x=0 wall
    mb.add_quad(P(X, 0, 0), P(X, 0, Z), P(X, Y, Z), P(X, Y, 0), mat)    # x=X wall


def interior(seed=0, spheres=180, level=2):
    """Plain-BDPT interior: closed 20x10x30 room, ``spheres`` icospheres of
    radius U[0.2,1.5] resting on the floor with vertices jittered by
    N(0, 0.02 r), one 2x2 ceiling light of radiance 20.  Level-2 icospheres
    (320 triangles) give 57,614 triangles in total."""
    rng = np.random.Generator(np.random.PCG64(seed))
    mb = MeshBuilder()
    wall = mb.add_material(material((0.7, 0.7, 0.7), specular=0.5, roughness=0.9))
    light = mb.add_material(material((0.8, 0.8, 0.8), emissive=(20.0, 20.0, 20.0), specular=0.0, roughness=1.0))
    X, Y, Z = 20.0, 10.0, 30.0
    _room(mb, X, Y, Z, wall)
    y = Y - 0.001
    mb.add_quad((9, y, 14), (11, y, 14), (11, y, 16), (9, y, 16), light)
    sv, sf = _icosphere(level)
    for _ in range(spheres):
        r = 0.2 + 1.3 * rng.random()
        cx = r + (X - 2 * r) * rng.random()
        cz = r + (Z - 2 * r) * rng.random()
        v = sv * r + (_gauss(rng, (len(sv), 3)) * 0.02 * r)
        v = v + np.array([cx, r, cz])
        m = mb.add_material(_disney(rng))
        mb.add_tris(v[sf], m)
    cam = dict(pos=(10.0, 5.0, 28.5), dir=(0.0, -0.25, -1.0), up=(0.0, 1.0, 0.0), fov=math.radians(60.0))
    return mb.build(), cam


def _grid_face(a, b, d, nu, nv):
    """Quad a,b,c=a+(b-a)+(d-a),d split into an nu x nv grid; returns (nu*nv*2,3,3)."""
    a, b, d = map(np.asarray, (a, b, d))
    ux, vx = (b - a) / nu, (d - a) / nv
    tris = []
    for i in range(nu):
        for j in range(nv):
            p00 = a + ux * i + vx * j
            p10 = p00 + ux
            p01 = p00 + vx
            p11 = p00 + ux + vx
            tris += [[p00, p10, p11], [p00, p11, p01]]
    return np.array(tris)


def _displaced_box(rng, cx, cz, sx, sy, sz, ang, amp):
    """Box tessellated to 200 triangles (four 5x2 side grids, two 5x6 caps),
    each grid vertex displaced by U[-amp, amp] on every axis."""
    cn = _box_corners(cx, cz, sx, sy, sz, ang)
    faces = _box_faces(cn)
    tris = []
    for k, (a, b, c, d) in enumerate(faces):
        nu, nv = (5, 6) if k < 2 else (5, 2)
        tris.append(_grid_face(a, b, d, nu, nv))
    tris = np.concatenate(tris)
    # displace shared grid points consistently: key on rounded position
    flat = tris.reshape(-1, 3)
    keys = np.round(flat * 1e5).astype(np.int64)
    uniq, inv = np.unique(keys, axis=0, return_inverse=True)
    disp = (rng.random((len(uniq), 3)) * 2.0 - 1.0) * amp
    flat = flat + disp[inv.reshape(-1)]
    return flat.reshape(-1, 3, 3)


def hall(seed=0, boxes=1200, pillar_rings=5):
    """Adaptive-BDPT hall: 40x8x40 room, 12x12 pillars (64-segment cylinders
    of radius 0.4 and height 8 in ``pillar_rings`` rings), ``boxes`` displaced
    boxes of 200 triangles, 4 ceiling lights of radiance U[5,30].
    332,180 triangles with the defaults."""
    rng = np.random.Generator(np.random.PCG64(seed))
    mb = MeshBuilder()
    wall = mb.add_material(material((0.7, 0.7, 0.7), specular=0.5, roughness=0.9))
    X, Y, Z = 40.0, 8.0, 40.0
    _room(mb, X, Y, Z, wall)
    y = Y - 0.001
    for (lx, lz) in ((10, 10), (30, 10), (10, 30), (30, 30)):
        rad = 5.0 + 25.0 * rng.random()
        lm = mb.add_material(material((0.8, 0.8, 0.8), emissive=(rad, rad, rad), specular=0.0, roughness=1.0))
        mb.add_quad((lx - 1, y, lz - 1), (lx + 1, y, lz - 1), (lx + 1, y, lz + 1), (lx - 1, y, lz + 1), lm)
    seg = 64
    ang = np.arange(seg + 1) * (2 * math.pi / seg)
    cs, sn = np.cos(ang), np.sin(ang)
    cs[-1], sn[-1] = cs[0], sn[0]
    for i in range(12):
        for j in range(12):
            cx, cz = (i + 0.5) * X / 12, (j + 0.5) * Z / 12
            m = mb.add_material(_disney(rng))
            tris = []
            for k in range(pillar_rings):
                y0, y1 = Y * k / pillar_rings, Y * (k + 1) / pillar_rings
                for s in range(seg):
                    p0 = (cx + 0.4 * cs[s], y0, cz + 0.4 * sn[s])
                    p1 = (cx + 0.4 * cs[s + 1], y0, cz + 0.4 * sn[s + 1])
                    p2 = (cx + 0.4 * cs[s + 1], y1, cz + 0.4 * sn[s + 1])
                    p3 = (cx + 0.4 * cs[s], y1, cz + 0.4 * sn[s])
                    tris += [[p0, p2, p1], [p0, p3, p2]]
            mb.add_tris(tris, m)
    for _ in range(boxes):
        sx, sy, sz = 0.3 + 0.9 * rng.random(3)
        cx = 0.5 + (X - 1.0) * rng.random()
        cz = 0.5 + (Z - 1.0) * rng.random()
        a = 2 * math.pi * rng.random()
        m = mb.add_material(_disney(rng))
        mb.add_tris(_displaced_box(rng, cx, cz, sx, sy, sz, a, 0.02 * min(sx, sy, sz)), m)
    cam = dict(pos=(20.0, 4.0, 39.0), dir=(0.0, -0.15, -1.0), up=(0.0, 1.0, 0.0), fov=math.radians(60.0))
    return mb.build(), cam


# Benchmark configurations (sizes from the workload definitions).
CONFIGS = {
    "cornell": dict(scene=cornell, width=256, height=256, spp=16, eye_depth=8, mode=0),
    "interior": dict(scene=interior, width=1024, height=768, spp=64, eye_depth=10, mode=0),
    "hall": dict(scene=hall, width=1280, height=720, spp=32, eye_depth=5, mode=1),
}
