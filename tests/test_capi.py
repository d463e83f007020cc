"""The C ABI library loads and exports every entry point include/gbpt.h declares (CPU only)."""
import ctypes
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "gbpt.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbpt_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_all_declared_symbols(gb):
    L = gb._native.load()
    names = _declared()
    assert len(names) >= 25
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(gb._native.SIGNATURES), set(names) ^ set(gb._native.SIGNATURES)


def test_struct_layouts_match_header(gb):
    from cudapt_gb300 import layouts
    assert layouts.VERTEX.itemsize == 44 and layouts.TRIANGLE.itemsize == 16 and layouts.MATERIAL.itemsize == 80
    L = gb._native.load()
    p = np.zeros((), layouts.PARAMS)
    gb._native.check(L.gbpt_params_default(p.ctypes.data))
    ref = layouts.default_params()
    assert p.tobytes() == ref.tobytes()


def test_host_side_errors_without_gpu(gb):
    import cudapt_gb300 as g
    from cudapt_gb300 import scenes
    (v, t, m), cam = scenes.cornell()
    bad = t.copy()
    bad["mat"][3] = 99
    try:
        g.RTScene(v, bad, m)
        raise AssertionError("expected GbptError")
    except g.GbptError as e:
        assert e.status == 1 and "material" in str(e)
    s = g.RTScene(v, t, m)
    info = s.bvh_info()
    assert info["nodes"] == 0 and info["tris"] == 36
    s.build_bvh()
    assert s.bvh_info()["nodes"] > 0 and s.bvh_info()["lights"] == 2


def test_gaussian_table_matches_oracle(gb, orc):
    L = gb._native.load()
    for delta, r in ((50.0, 5), (3.0, 4), (0.7, 9)):
        g = np.zeros(64, np.float32)
        gb._native.check(L.gbpt_gaussian_table(delta, r, g.ctypes.data))
        want = orc.gaussian(delta, r)
        assert np.array_equal(g[: 2 * r + 1].view(np.uint32), want[: 2 * r + 1].view(np.uint32))
