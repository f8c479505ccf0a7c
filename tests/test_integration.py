"""The reference-side adapter shown in INTEGRATION.md (render_gpu over
lajolla's own Scene types) compiles against the reference's headers and the
C ABI header.  Needs the reference sources, so it runs in the development
container only (skipped elsewhere)."""
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = "/root/reference"


def adapter_source():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    section = text.split("## C++: the adapter", 1)[1]
    m = re.search(r"```cpp\n(.*?)```", section, flags=re.S)
    return m.group(1)


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")), reason="reference sources not present")
def test_adapter_compiles_against_reference_headers():
    src = adapter_source()
    assert "render_gpu(const Scene &scene)" in src
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "render_gpu.cpp")
        open(f, "w").write(src)
        r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-w", "-I", os.path.join(REF, "src"),
                            "-I", os.path.join(REF, "embree", "include"), "-I", os.path.join(ROOT, "include"), f],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
