"""The reference-side binding shown in INTEGRATION.md (camera_gpu.h, a
device backend for camera::render) compiles against the reference's own
headers and this backend's C ABI header, and links against the library.
Needs the reference checkout (REFERENCE, as tests/golden/gen_golden.py
reads it); skipped where it is absent."""
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REFERENCE = os.environ.get("REFERENCE", "/root/reference")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE, "include")), reason="no reference checkout")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_integration_snippet_builds(tmp_path):
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    m = re.search(r"```cpp\n(// camera_gpu\.h.*?)```", text, re.S)
    assert m, "the binding snippet is missing"
    (tmp_path / "camera_gpu.h").write_text(m.group(1))
    (tmp_path / "main.cpp").write_text(
        '#include "camera_gpu.h"\n'
        "int main(int argc, char** argv) {\n"
        "    if (argc < 2) return 0;\n"
        "    camera cam;\n"
        "    frame f = render_device(argv[1], cam, 0, nullptr);\n"
        "    return f.radiance.empty() ? 1 : 0;\n"
        "}\n")
    lib_dir = os.path.join(ROOT, "mypbr_gb300", "_lib")
    cmd = ["g++", "-std=c++17", "-O0", "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(REFERENCE, "include"),
           "-isystem", os.path.join(REFERENCE, "external"), "-I" + str(tmp_path), str(tmp_path / "main.cpp"),
           "-L" + lib_dir, "-lmypbr_gb300", "-Wl,-rpath," + lib_dir, "-lpthread", "-o", str(tmp_path / "render_gpu")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    # without arguments it exits at once: the binary loads the library
    assert subprocess.run([str(tmp_path / "render_gpu")]).returncode == 0
