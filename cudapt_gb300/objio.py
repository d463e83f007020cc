"""Small OBJ + MTL reader producing CudaPT's scene records.

Stands in for the Assimp import of ``RTScene::AddModel``
(src/raytracer.cpp:98-237): positions, normals and texture coordinates per
face corner, polygons split into fans (aiProcess_Triangulate), flat normals
when the file has none (aiProcess_GenNormals), and materials converted as
``AssimpProcessSceneMaterial`` does (src/raytracer.cpp:208-234):

* diffuse = Kd, emissive = Ka + Ke (the reference adds the ambient colour
  into the emissive one), transparency = 1 - d;
* everything else keeps the RTMaterial defaults (include/raytracer.h:110-124).

Faces stay in file order; Assimp's per-material mesh splitting is not
reproduced.  Texture maps are not loaded (texture ids stay -1).
"""
import os

import numpy as np

from .layouts import MATERIAL, TRIANGLE, VERTEX, material


def _mtl(path):
    mats, cur = {}, None
    if not os.path.exists(path):
        return mats
    with open(path, errors="replace") as f:
        for line in f:
            p = line.split()
            if not p or p[0].startswith("#"):
                continue
            k = p[0]
            if k == "newmtl":
                cur = " ".join(p[1:])
                mats[cur] = {}
            elif cur is not None and k in ("Kd", "Ka", "Ke") and len(p) >= 4:
                mats[cur][k] = tuple(float(x) for x in p[1:4])
            elif cur is not None and k in ("d", "Tr") and len(p) >= 2:
                mats[cur][k] = float(p[1])
    return mats


def _to_material(d):
    m = material(diffuse=d.get("Kd", (1.0, 1.0, 1.0)), emissive=(0.0, 0.0, 0.0))
    ka = np.array(d.get("Ka", (0.0, 0.0, 0.0)), np.float32)
    ke = np.array(d.get("Ke", (0.0, 0.0, 0.0)), np.float32)
    m["emissive"] = ka + ke
    if "d" in d:
        m["transparency"] = 1.0 - d["d"]
    elif "Tr" in d:
        m["transparency"] = d["Tr"]
    return m


def load_obj(path, with_materials=True, default=None):
    """Return (vertices, triangles, materials) record arrays."""
    pos, nrm, tex = [], [], []
    corners, cnorm, ctex, fmat = [], [], [], []
    mtl, names, cur = {}, [], None
    base = os.path.dirname(path)
    with open(path, errors="replace") as f:
        for line in f:
            p = line.split()
            if not p or p[0].startswith("#"):
                continue
            k = p[0]
            if k == "v":
                pos.append([float(x) for x in p[1:4]])
            elif k == "vn":
                nrm.append([float(x) for x in p[1:4]])
            elif k == "vt":
                tex.append([float(x) for x in p[1:3]] + [0.0] * (2 - len(p[1:3])))
            elif k == "mtllib" and with_materials:
                mtl.update(_mtl(os.path.join(base, " ".join(p[1:]))))
            elif k == "usemtl":
                cur = " ".join(p[1:])
                if cur not in names:
                    names.append(cur)
            elif k == "f":
                idx = []
                for c in p[1:]:
                    parts = c.split("/")
                    vi = int(parts[0])
                    ti = int(parts[1]) if len(parts) > 1 and parts[1] else 0
                    ni = int(parts[2]) if len(parts) > 2 and parts[2] else 0
                    vi = vi - 1 if vi > 0 else len(pos) + vi
                    ti = (ti - 1 if ti > 0 else len(tex) + ti) if ti else -1
                    ni = (ni - 1 if ni > 0 else len(nrm) + ni) if ni else -1
                    idx.append((vi, ti, ni))
                mid = names.index(cur) if cur in names else -1
                for j in range(1, len(idx) - 1):  # fan
                    tri = (idx[0], idx[j], idx[j + 1])
                    corners.append([c[0] for c in tri])
                    ctex.append([c[1] for c in tri])
                    cnorm.append([c[2] for c in tri])
                    fmat.append(mid)
    P = np.array(pos, np.float32)
    C = np.array(corners, np.int64).reshape(-1, 3)
    T = len(C)
    verts = np.zeros(T * 3, VERTEX)
    tp = P[C]  # (T,3,3)
    verts["pos"] = tp.reshape(-1, 3)
    e0 = (tp[:, 1] - tp[:, 0]).astype(np.float64)
    e1 = (tp[:, 2] - tp[:, 0]).astype(np.float64)
    fn = np.cross(e0, e1)
    ln = np.linalg.norm(fn, axis=1, keepdims=True)
    ln[ln == 0] = 1.0
    fn = (fn / ln).astype(np.float32)
    N = np.array(nrm, np.float32) if nrm else np.zeros((0, 3), np.float32)
    CN = np.array(cnorm, np.int64).reshape(-1, 3)
    vn = np.repeat(fn, 3, axis=0).reshape(T, 3, 3)
    has = CN >= 0
    if len(N):
        vn[has] = N[CN[has]]
    verts["norm"] = vn.reshape(-1, 3)
    if tex:
        TX = np.array(tex, np.float32)
        CT = np.array(ctex, np.int64).reshape(-1, 3)
        uv = np.zeros((T, 3, 2), np.float32)
        ht = CT >= 0
        uv[ht] = TX[CT[ht]]
        uv[..., 1] = 1.0 - uv[..., 1]  # aiProcess_FlipUVs
        verts["tex"] = uv.reshape(-1, 2)
    tris = np.zeros(T, TRIANGLE)
    ids = np.arange(T * 3, dtype=np.uint32).reshape(T, 3)
    tris["v0"], tris["v1"], tris["v2"] = ids[:, 0], ids[:, 1], ids[:, 2]
    mats = [_to_material(mtl.get(n, {})) if with_materials else (default if default is not None else material())
            for n in names] or [default if default is not None else material()]
    fm = np.array(fmat, np.int64)
    fm[fm < 0] = 0
    if not with_materials:
        fm[:] = 0
        mats = mats[:1]
    tris["mat"] = fm.astype(np.uint32)
    return verts, tris, np.array(mats, MATERIAL).reshape(-1)
