"""The benchmark's byte model (CPU): bench.py's per-class algorithmic bytes
equal the constants and formulas of include/lj_bytes_model.h, compiled here
with the host C compiler, so the roofline numerator has one definition."""
import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

NAMES = ["LJ_BYTES_RAY", "LJ_BYTES_HIT", "LJ_BYTES_PATH_STATE", "LJ_BYTES_SHADE_GEOM",
         "LJ_BYTES_SHADE_MATERIAL", "LJ_BYTES_SHADOW_ENTRY", "LJ_BYTES_VOL_STATE",
         "LJ_BYTES_NEE_REQUEST", "LJ_BYTES_NEE_RESULT", "LJ_BYTES_VOL_SEGMENT",
         "LJ_BYTES_NEE_SHADOW_LOOP", "LJ_BYTES_SHADE_SEGMENT",
         "LJ_BYTES_TRACE_CLOSEST(0)", "LJ_BYTES_TRACE_SHADOW(0)"]


def header_values(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "bm.c"
    body = "".join('    printf("%%ld\\n", (long)(%s));\n' % n for n in NAMES)
    src.write_text('#include <stdio.h>\n#include "lj_bytes_model.h"\nint main(void) {\n%s    return 0;\n}\n'
                   % body)
    exe = tmp_path / "bm"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    return dict(zip(NAMES, map(int, out)))


def test_bench_byte_model_matches_header(tmp_path):
    import bench
    from lajolla_public_gb300 import abi
    h = header_values(tmp_path)
    assert h["LJ_BYTES_RAY"] == bench.BYTES_RAY
    assert h["LJ_BYTES_HIT"] == bench.BYTES_HIT
    assert h["LJ_BYTES_PATH_STATE"] == bench.BYTES_PATH_STATE
    assert h["LJ_BYTES_SHADE_GEOM"] == bench.BYTES_SHADE_GEOM
    assert h["LJ_BYTES_SHADE_MATERIAL"] == bench.BYTES_SHADE_MAT
    assert h["LJ_BYTES_SHADOW_ENTRY"] == bench.BYTES_SHADOW_ENTRY
    assert h["LJ_BYTES_VOL_STATE"] == bench.BYTES_VOL_STATE
    assert h["LJ_BYTES_NEE_REQUEST"] == bench.BYTES_NEE_REQUEST
    assert h["LJ_BYTES_NEE_RESULT"] == bench.BYTES_NEE_RESULT
    assert h["LJ_BYTES_VOL_SEGMENT"] == bench.BYTES_VOL_SEGMENT
    assert h["LJ_BYTES_NEE_SHADOW_LOOP"] == bench.BYTES_NEE_SHADOW_LOOP
    # one unit of each class through bench.kernel_bytes
    kb = bench.kernel_bytes
    assert kb(abi.LJ_KERNEL_TRACE, 0, 1, 0, 0) == h["LJ_BYTES_TRACE_CLOSEST(0)"]
    assert kb(abi.LJ_KERNEL_SHADOW, 0, 0, 1, 0) == h["LJ_BYTES_TRACE_SHADOW(0)"]
    assert kb(abi.LJ_KERNEL_SHADE, 0, 0, 0, 1) == h["LJ_BYTES_SHADE_SEGMENT"]
    assert kb(abi.LJ_KERNEL_SHADE, 0, 0, 1, 1) == h["LJ_BYTES_SHADE_SEGMENT"] + h["LJ_BYTES_SHADOW_ENTRY"]
    assert kb(abi.LJ_KERNEL_MEDIUM, 0, 0, 0, 0, vol_segments=1) == h["LJ_BYTES_VOL_SEGMENT"]
    assert kb(abi.LJ_KERNEL_NEE, 0, 0, 0, 0, nee_requests=1) == h["LJ_BYTES_NEE_SHADOW_LOOP"]
    assert kb(abi.LJ_KERNEL_OTHER, 1, 1, 1, 1, 1, 1) == 0
