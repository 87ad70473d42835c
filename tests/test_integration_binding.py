"""The reference-side binding (include/camera_gpu.h, a device backend for
camera::render) compiles against the reference's own headers and this
backend's C ABI header, links against the library together with the
reference's load_scene, and the program loads. Needs the reference checkout
(oracle/Makefile knows where it lies); skipped where it is absent."""
import os
import shutil
import subprocess

import pytest

from mypbr_gb300 import build

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REFERENCE = build.reference_dir()


@pytest.mark.skipif(REFERENCE is None, reason="no reference checkout")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_reference_binding_builds(tmp_path):
    stb = os.path.join(ROOT, "oracle", "_ref", "stb_impl.o")
    assert os.path.exists(stb), "build the reference harness first (make -C oracle ref)"
    (tmp_path / "main.cpp").write_text(
        '#include "scene.h"\n'
        '#include "camera_gpu.h"\n'
        "int main(int argc, char** argv) {\n"
        "    if (argc < 2) return 0;\n"
        "    scene sc;\n"
        "    if (!load_scene(argv[1], sc)) return 2;\n"
        "    frame f = render_device(argv[1], sc.cam, 0, nullptr);\n"
        "    return f.radiance.empty() ? 1 : 0;\n"
        "}\n")
    lib_dir = os.path.join(ROOT, "mypbr_gb300", "_lib")
    cmd = ["g++", "-std=c++17", "-O0", "-Wall", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(REFERENCE, "include"), "-isystem", os.path.join(REFERENCE, "external"),
           str(tmp_path / "main.cpp"), stb, "-L" + lib_dir, "-lmypbr_gb300", "-Wl,-rpath," + lib_dir, "-lpthread",
           "-o", str(tmp_path / "render_gpu")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    # without arguments it exits at once: the binary loads the library
    assert subprocess.run([str(tmp_path / "render_gpu")]).returncode == 0
