"""The C++ RTScene / RTRenderer shim (include/gbpt.hpp) compiles against the
C ABI and links libgbpt.so; without a GPU the device check reports so."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r"""
#include "gbpt.hpp"
#include <cstdio>
int main() {
  int32_t ok = -1;
  gbpt_status s = gbpt_device_check(&ok);
  gbpt::RTScene scene;
  scene.m_pVertices.resize(3);
  scene.m_pTriangles.push_back(gbpt_triangle{0, 1, 2, 0});
  scene.m_pMaterials.resize(1);
  for (int i = 0; i < 3; i++) scene.m_pVertices[i].pos[0] = (float)i;
  bool threw = false;
  try {
    gbpt::RTRenderer r;
    r.SetRendererMode(GBPT_MODE_BDPT_SC_BILAT);
    (void)r.GetRendererMode();
    scene.UpdateBVH();
  } catch (const gbpt::Error& e) {
    threw = true;
  }
  std::printf("%d %d %d\n", (int)s, ok, threw ? 1 : 0);
  return 0;
}
"""


def test_cpp_shim_compiles_and_links(tmp_path):
    from cudapt_gb300 import build
    lib = build.build()
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    src = tmp_path / "shim.cpp"
    src.write_text(SRC)
    exe = tmp_path / "shim"
    subprocess.run([gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    "-L", os.path.dirname(lib), "-lgbpt", "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    status, ok, threw = (int(x) for x in out.stdout.split())
    assert status in (0, 7)  # GBPT_OK with a device, GBPT_ERR_NO_DEVICE without
    if status == 7:
        assert ok == 0
