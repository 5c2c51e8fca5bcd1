"""Drop-in checks that need no GPU.

* The reference's own fluidtest sources (test/src/main.cpp and
  test/src/myfluidsystem.cpp) compile unchanged against include/fluidsystem.h
  and link with libfluid.so (oracle/ref_fluidtest.sh; skipped where the
  reference tree is absent).
* sph_write_geo produces byte-identical .geo files to the reference's own
  dumpToGeo (test/src/main.cpp:10-74), linked into oracle/_ref/geo_check.
* include/fluidsystem.h is self-contained C++ (a subclass in the style of
  test/src/myfluidsystem.h compiles and links).
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_ROOT = os.environ.get("LIBFLUID_REFERENCE", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "test", "src", "main.cpp")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


@pytest.mark.skipif(not os.path.exists(REF_SRC), reason="reference tree not present")
def test_reference_fluidtest_compiles_and_geo_matches(tmp_path):
    r = subprocess.run(["bash", os.path.join(ROOT, "oracle", "ref_fluidtest.sh"), REF_ROOT], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert os.path.exists(os.path.join(ROOT, "oracle", "_ref", "ref_fluidtest"))
    g = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "geo_check"), str(tmp_path)], capture_output=True,
                       text=True)
    assert g.returncode == 0, g.stdout + g.stderr
    assert "identical" in g.stdout


def test_dropin_header_subclass_compiles(tmp_path):
    src = tmp_path / "sub.cpp"
    src.write_text(
        '#include "fluidsystem.h"\n'
        "class MyFluidSystem : public FluidSystem {\n"
        "public:\n"
        "  void setupDoubleDamBreak(const uint &n, const uint &res) {\n"
        "    init(n, res); setAdhesion(0.1f); setViscosity(0.2f); setSurfaceTension(1.0f); setVDamp(0.5f);\n"
        "    createFluidBlock(0, n / 2, 0.0, 0.0, 0.0, 0.33, 0.9, 0.33);\n"
        "    createFluidBlock(n / 2, n - n / 2, 0.66f, 0.0f, 0.66f, 1.0f, 0.9f, 1.0f);\n"
        "    if (!m_isInit) clear();\n"
        "  }\n"
        "};\n"
        "int main() { MyFluidSystem s; std::vector<float3> p(4), c(4), v(4);\n"
        "  if (s.getPscale() < 0) { s.setupDoubleDamBreak(4, 8); s.advance(); s.advance(0.002f, 1);\n"
        "    s.exportToData(p, c, v); s.setupFromData(p, v); s.setup(4, 8); }\n"
        "  return FluidSystem::DYNAMIC == 2 ? 0 : 1; }\n")
    exe = tmp_path / "sub"
    r = subprocess.run(["g++", "-std=c++11", f"-I{os.path.join(ROOT, 'include')}", f"-I{CUDA}/include", str(src),
                        "-o", str(exe), f"-L{os.path.join(ROOT, 'libfluid_gb300')}", "-lfluid", "-lsph_gb300",
                        f"-Wl,-rpath,{os.path.join(ROOT, 'libfluid_gb300')}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_geo_path_format():
    import ctypes as C
    from libfluid_gb300 import _capi
    buf = C.create_string_buffer(64)
    assert _capi.lib().sph_geo_path(buf, 64, b"geo/sim", 7) == 0
    assert buf.value == b"geo/sim.0007.geo"
    assert _capi.lib().sph_geo_path(buf, 8, b"geo/sim", 7) != 0
