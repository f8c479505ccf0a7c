"""C-ABI checks that need no GPU: the library builds and loads, it exports
every function include/lj_gpu.h declares, and the ctypes mirror has the C
struct sizes."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from lajolla_public_gb300 import abi, build, gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", h) for h in sorted(os.listdir(os.path.join(ROOT, "include")))
           if h.endswith(".h")]


def declared_functions():
    names = []
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*?\*?\s*\*?\s*(lj_gpu_[a-z0-9_]+)\s*\(",
                             text, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


def test_library_builds_and_loads():
    path = build.build()
    assert os.path.exists(path)
    L = gpu.lib()
    assert L.lj_gpu_abi_version() == abi.LJ_GPU_ABI_VERSION == 4


def test_every_declared_symbol_is_exported():
    names = declared_functions()
    assert len(names) >= 15, names
    L = gpu.lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_every_binding_declares_the_header_parameter_count():
    """gpu.lib() gives every declared function ctypes argument types, as many
    as the header's prototype has (an undeclared pointer argument would be
    passed as a 32-bit int)."""
    L = gpu.lib()
    protos = {}
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"\b(lj_gpu_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
            args = m.group(2).strip()
            protos[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    assert set(protos) == set(declared_functions())
    bad = [(n, k, getattr(L, n).argtypes) for n, k in sorted(protos.items())
           if getattr(L, n).argtypes is None or len(getattr(L, n).argtypes) != k]
    assert not bad, bad


def test_struct_sizes_match_c():
    names = sorted(abi.STRUCT_SIZES)
    src = "#include <stdio.h>\n#include \"lj_gpu.h\"\nint main(void){\n"
    for n in names:
        src += '  printf("%%s %%zu\\n", "%s", sizeof(%s));\n' % (n, n)
    src += "  return 0;\n}\n"
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "s.c")
        exe = os.path.join(d, "s")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    sizes = dict((l.split()[0], int(l.split()[1])) for l in out.splitlines())
    for n in names:
        assert sizes[n] == abi.STRUCT_SIZES[n], (n, sizes[n], abi.STRUCT_SIZES[n])


def test_struct_field_offsets_match_c():
    """Every field of every ctypes mirror sits at the C compiler's offset (a
    size match alone would miss two swapped fields of one size)."""
    fields = []
    for n in sorted(abi.STRUCT_SIZES):
        cls = getattr(abi, n)
        for f in cls._fields_:
            fields.append((n, f[0], getattr(cls, f[0]).offset))
    src = "#include <stdio.h>\n#include <stddef.h>\n#include \"lj_gpu.h\"\nint main(void){\n"
    for n, f, _ in fields:
        src += '  printf("%%zu\\n", offsetof(%s, %s));\n' % (n, f)
    src += "  return 0;\n}\n"
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "o.c")
        exe = os.path.join(d, "o")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    assert len(out) == len(fields) > 50
    bad = [(n, f, py, int(c)) for (n, f, py), c in zip(fields, out) if py != int(c)]
    assert not bad, bad


def test_constants_match_c():
    """Every LJ_ integer constant of the ctypes mirror (error codes, kinds,
    kernel classes, the ABI version) has the header's value, and the mirror
    names every constant the header defines."""
    text = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "lj_gpu.h")).read(), flags=re.S)
    in_header = set(re.findall(r"\b(LJ_[A-Z0-9_]+)\b", text)) - {"LJ_GPU_H"}
    names = sorted(k for k in dir(abi) if k.startswith("LJ_") and isinstance(getattr(abi, k), int))
    assert set(names) == in_header, sorted(set(names) ^ in_header)
    src = "#include <stdio.h>\n#include \"lj_gpu.h\"\nint main(void){\n"
    for n in names:
        src += '  printf("%%lld\\n", (long long)(%s));\n' % n
    src += "  return 0;\n}\n"
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "k.c")
        exe = os.path.join(d, "k")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    bad = [(n, getattr(abi, n), int(v)) for n, v in zip(names, out) if getattr(abi, n) != int(v)]
    assert not bad, bad


def test_init_without_gpu_fails_loudly():
    """No CPU fallback: without a CUDA device the context cannot be created."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gpu.LjError):
        gpu.Context(0)


def test_bsdf_param_counts_match_python_layout():
    L = gpu.lib()
    for t in range(abi.LJ_MAT_COUNT):
        assert L.lj_gpu_bsdf_param_count(t) == abi.BSDF_PARAM_COUNT[t]
        assert sum(abi.SLOT_WIDTHS[t]) + 1 == abi.BSDF_PARAM_COUNT[t]
    assert L.lj_gpu_bsdf_param_count(99) == -1
