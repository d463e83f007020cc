"""Reader and writer of CudaPT's ``.NPRTENV`` environment presets.

Restates ``CUDAPTWindow::BrowseEnvSetting`` / ``BrowseAndSaveEnvSetting``
(src/cudapt.cpp:623-836) and the token reader ``txtConfFile``
(src/conffilehelper.cpp:32-115): a whitespace-separated stream of
``name value...`` records, ``//`` comments to the end of the line and
``/* */`` block comments.  Records:

* ``campos x y z`` and ``campitchyaw pitch yaw`` -- the fly camera
  (include/camhelper.h:142-240): direction (cos(yaw) sin(pitch), sin(yaw),
  cos(yaw) cos(pitch)) normalised, up (0, 1, 0), fov pi/4 (src/cudapt.cpp:388);
* ``rttech n`` -- the renderer's index in RTRenderer::RENDERER_MODE;
* ``models n path...`` -- model files, relative to the working directory;
* ``materials n`` + 19 numbers per material in the reference's order
  (anisotropic, clearcoat, clearcoatGloss, diffuse[3], diffuseTexId,
  emissive[3], emissiveTexId, metallic, normalTexId, roughness, sheen,
  sheenTint, specular, subsurface, transparency);
* ``convergedresult`` + W*H*3 floats -- the reference image of the RMSE
  experiments (src/cudapt.cpp:951-997).
"""
import math
import re

import numpy as np

from .layouts import (MATERIAL, MODE_BDPT_SC, MODE_BDPT_SC_ADAP_BILAT, MODE_BDPT_SC_ADAP_BILAT_BINARY,
                      MODE_BDPT_SC_BILAT, MODE_PT_SC)

# RTRenderer::RENDERER_MODE with FULLSPECTRAL off (include/raytracer.h:1-26,
# 295-304): CPU debug, then the X-macro entries in order.
RTTECH_NAMES = ["CPU Debug", "RasterizeBasic", "PTNaive", "PTSC", "BDPTRegen", "BDPTSC", "BDPTSC Bilaterial",
                "BDPTSC Adap Bilat Binary", "BDPTSC Adap Bilat PLL", "BDPTSA Adap Bilat PLL", "Cuda Debug",
                "Cuda BVH Debug"]
RTTECH_TO_MODE = {3: MODE_PT_SC, 5: MODE_BDPT_SC, 6: MODE_BDPT_SC_BILAT, 7: MODE_BDPT_SC_ADAP_BILAT_BINARY,
                  8: MODE_BDPT_SC_ADAP_BILAT, 9: MODE_BDPT_SC_ADAP_BILAT}
MODE_TO_RTTECH = {MODE_PT_SC: 3, MODE_BDPT_SC: 5, MODE_BDPT_SC_BILAT: 6, MODE_BDPT_SC_ADAP_BILAT_BINARY: 7,
                  MODE_BDPT_SC_ADAP_BILAT: 8}

_MAT_FIELDS = [("anisotropic", 1), ("clearcoat", 1), ("clearcoatGloss", 1), ("diffuse", 3), ("diffuseTexId", 1),
               ("emissive", 3), ("emissiveTexId", 1), ("metallic", 1), ("normalTexId", 1), ("roughness", 1),
               ("sheen", 1), ("sheenTint", 1), ("specular", 1), ("subsurface", 1), ("transparency", 1)]
MAT_WORDS = sum(n for _, n in _MAT_FIELDS)  # 19


def _tokens(text):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", " ", text)
    return text.split()


def fly_camera(pos, pitch, yaw):
    """FlyCamera::GetDir / GetUp (include/camhelper.h:201-214), fov M_PI_2 * 0.5."""
    c = math.cos(yaw)
    d = np.array([c * math.sin(pitch), math.sin(yaw), c * math.cos(pitch)], np.float64)
    d = d / np.linalg.norm(d)
    return dict(pos=tuple(float(x) for x in pos), dir=tuple(float(x) for x in d), up=(0.0, 1.0, 0.0),
                fov=math.pi / 4)


def load(path, width=None, height=None):
    """Parse a preset file; returns a dict with the records found."""
    with open(path, errors="replace") as f:
        tok = _tokens(f.read())
    out = {"models": [], "materials": None, "converged": None}
    i = 0

    def take(n):
        nonlocal i
        v = tok[i:i + n]
        if len(v) < n:
            raise ValueError(f"{path}: truncated record")
        i += n
        return v

    while i < len(tok):
        name = tok[i]
        i += 1
        if name == "campos":
            out["campos"] = tuple(float(x) for x in take(3))
        elif name == "campitchyaw":
            out["pitch"], out["yaw"] = (float(x) for x in take(2))
        elif name == "rttech":
            out["rttech"] = int(take(1)[0])
        elif name == "models":
            n = int(take(1)[0])
            out["models"] = take(n)
        elif name == "materials":
            n = int(take(1)[0])
            mats = np.zeros(n, MATERIAL)
            for k in range(n):
                vals = take(MAT_WORDS)
                j = 0
                for fname, cnt in _MAT_FIELDS:
                    v = [float(x) for x in vals[j:j + cnt]]
                    mats[k][fname] = v if cnt > 1 else v[0]
                    j += cnt
            out["materials"] = mats
        elif name == "convergedresult":
            if width is None or height is None:
                raise ValueError("convergedresult needs the image size")
            out["converged"] = np.array([float(x) for x in take(width * height * 3)], np.float32)
        # unknown names are skipped, as the reference's reader does
    if "campos" in out and "pitch" in out:
        out["camera"] = fly_camera(out["campos"], out["pitch"], out["yaw"])
    if "rttech" in out:
        out["mode"] = RTTECH_TO_MODE.get(out["rttech"])
    return out


def _num(x):
    return format(float(x), "g") if not float(x).is_integer() else str(int(x)) if abs(x) < 1e15 else format(x, "g")


def save(path, campos, pitch, yaw, mode=MODE_BDPT_SC, models=(), materials=None, converged=None):
    """Write a preset in the reference's layout (BrowseAndSaveEnvSetting)."""
    lines = ["//\tRay Tracer Environment Setting File (Strict Format)", "//\tgbpt"]
    lines.append("campos\t" + "\t".join(_num(v) for v in campos))
    lines.append(f"campitchyaw\t{_num(pitch)}\t{_num(yaw)}")
    lines.append(f"rttech\t{MODE_TO_RTTECH.get(mode, 5)}")
    if models:
        lines.append("models\t" + str(len(models)) + "\t" + "\t".join(models))
    if materials is not None and len(materials):
        words = [str(len(materials))]
        for m in np.asarray(materials, MATERIAL).reshape(-1):
            for fname, cnt in _MAT_FIELDS:
                v = np.atleast_1d(m[fname])
                words += [_num(x) for x in v]
        lines.append("materials\t" + "\t".join(words))
    if converged is not None:
        lines.append("convergedresult\t" + "\t".join(format(float(x), ".9g") for x in np.asarray(converged).ravel()))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def apply_materials(scene_materials, preset_materials):
    """Overwrite the first n scene materials with the preset's (as the reference does when the scene has >= n)."""
    out = np.array(scene_materials, MATERIAL, copy=True)
    if preset_materials is None or len(out) < len(preset_materials):
        return out
    for name in MATERIAL.names:
        if name == "matType":
            continue
        out[name][: len(preset_materials)] = preset_materials[name]
    return out
