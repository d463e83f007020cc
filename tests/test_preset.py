""".NPRTENV presets (src/cudapt.cpp:623-836): the reference's own shipped
preset (copied to tests/golden/) parses, round-trips, and drives a scene."""
import math
import os

import numpy as np

from cudapt_gb300 import layouts, preset

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_reference_preset_parses():
    d = preset.load(os.path.join(GOLD, "cornellwtranball.NPRTENV"))
    assert d["campos"] == (-1.82495, -2.40754, -2.74389)
    assert (d["pitch"], d["yaw"]) == (-0.13, -0.215)
    assert d["rttech"] == 3 and preset.RTTECH_NAMES[3] == "PTSC" and d["mode"] == layouts.MODE_PT_SC
    assert d["models"] == ["..\\asset\\model\\cornell_box_with_sphere.obj"]
    m = d["materials"]
    assert len(m) == 6
    np.testing.assert_allclose(m[0]["diffuse"], [0.6, 0.6, 0.6])
    np.testing.assert_allclose(m[2]["emissive"], [20.0, 20.0, 20.0])  # the light
    assert m[0]["diffuseTexId"] == -1 and m[0]["normalTexId"] == -1
    cam = d["camera"]
    assert math.isclose(np.linalg.norm(cam["dir"]), 1.0, rel_tol=1e-12)
    assert cam["up"] == (0.0, 1.0, 0.0) and math.isclose(cam["fov"], math.pi / 4)


def test_round_trip(tmp_path):
    d = preset.load(os.path.join(GOLD, "cornellwtranball.NPRTENV"))
    conv = np.linspace(0, 1, 4 * 3 * 3, dtype=np.float32)
    p = tmp_path / "x.NPRTENV"
    preset.save(str(p), d["campos"], d["pitch"], d["yaw"], layouts.MODE_BDPT_SC_ADAP_BILAT, d["models"],
                d["materials"], conv)
    e = preset.load(str(p), width=4, height=3)
    assert e["campos"] == d["campos"] and (e["pitch"], e["yaw"]) == (d["pitch"], d["yaw"])
    assert e["mode"] == layouts.MODE_BDPT_SC_ADAP_BILAT and e["rttech"] == 8
    assert e["materials"].tobytes() == d["materials"].tobytes()
    np.testing.assert_array_equal(e["converged"], conv)


def test_comments_and_unknown_records(tmp_path):
    p = tmp_path / "c.NPRTENV"
    p.write_text("// header\ncampos 1 2 3 /* inline */ campitchyaw 0 0\nunknownrecord\nrttech 5 // bdpt\n")
    d = preset.load(str(p))
    assert d["campos"] == (1.0, 2.0, 3.0) and d["mode"] == layouts.MODE_BDPT_SC
    assert d["camera"]["dir"] == (0.0, 0.0, 1.0)


def test_apply_materials_to_scene():
    d = preset.load(os.path.join(GOLD, "cornellwtranball.NPRTENV"))
    g = np.load(os.path.join(GOLD, "obj_cornell.npz"))
    scene_mats = np.repeat(g["materials"], 6)
    out = preset.apply_materials(scene_mats, d["materials"])
    np.testing.assert_allclose(out["emissive"][2], [20.0, 20.0, 20.0])
    # fewer scene materials than the preset: left unchanged, as the reference does
    assert preset.apply_materials(scene_mats[:2], d["materials"]).tobytes() == scene_mats[:2].tobytes()
