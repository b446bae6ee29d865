"""The C ABI without a GPU: the library builds, loads and exports every entry
point include/bmxg.h declares, and the ctypes mirror has the C layout."""
import ctypes as C
import os
import re
import subprocess

import pytest

from boltzmannmfx_gb300 import abi, build, runtime

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
HEADER = os.path.join(ROOT, "include", "bmxg.h")


def declared_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(bmxg_[a-z_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return runtime.load_library()


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 13
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(runtime.ABI_SYMBOLS)


def test_version(lib):
    assert lib.bmxg_version() == 2


def test_create_without_device_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    h = C.c_void_p()
    p = abi.Params()
    g = abi.Geometry.make((0, 0, 0), (1, 1, 1), (4, 4, 4), (1, 1, 0))
    rc = lib.bmxg_create(C.byref(p), 1, C.byref(g), C.byref(h))
    assert rc == abi.BMXG_ERR_CUDA and not h.value


def test_struct_layout_matches_c(tmp_path):
    src = tmp_path / "layout.c"
    fields = {
        "bmxg_params": [f for f, _ in abi.Params._fields_],
        "bmxg_geometry": [f for f, _ in abi.Geometry._fields_],
        "bmxg_particles": [f for f, _ in abi.ParticlesStruct._fields_],
        "bmxg_stats": [f for f, _ in abi.Stats._fields_],
        "bmxg_shapes": [f for f, _ in abi.Shapes._fields_],
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "bmxg.h"', "int main(void){"]
    for st, fs in fields.items():
        lines.append(f'printf("{st} %zu\\n", sizeof({st}));')
        for f in fs:
            lines.append(f'printf("{st}.{f} %zu\\n", offsetof({st}, {f}));')
    lines.append("return 0;}")
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                         check=True).stdout.split("\n") if l)
    for st, cls in (("bmxg_params", abi.Params), ("bmxg_geometry", abi.Geometry),
                    ("bmxg_particles", abi.ParticlesStruct), ("bmxg_stats", abi.Stats),
                    ("bmxg_shapes", abi.Shapes)):
        assert int(out[st]) == C.sizeof(cls), st
        for f, _ in cls._fields_:
            assert int(out[f"{st}.{f}"]) == getattr(cls, f).offset, (st, f)


def test_constants_match_header():
    txt = open(HEADER).read()
    for name in ("BMXG_OK", "BMXG_ERR_ARG", "BMXG_ERR_CUDA", "BMXG_ERR_OOM", "BMXG_ERR_CAPACITY",
                 "BMXG_ERR_STATE", "BMXG_ERR_NONFINITE", "BMXG_ERR_TIMEOUT", "BMXG_ERR_UNSUPPORTED",
                 "BMXG_HOST", "BMXG_DEVICE", "BMXG_FP64", "BMXG_FP32F"):
        m = re.search(rf"#define {name}\s+(-?\d+)", txt)
        assert m and int(m.group(1)) == getattr(abi, name), name


def test_no_cpu_fallback_in_product():
    """The product never imports or links the oracle."""
    pkg = os.path.join(ROOT, "boltzmannmfx_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                txt = open(os.path.join(dirpath, f)).read()
                for pat in (r"^\s*(from|import)\s+oracle", r"liboracle", r"bmx_oracle", r"libbmxref",
                            r"orc_[a-z_]+\s*\("):
                    assert not re.search(pat, txt, re.M), (f, pat)


def test_particles_struct_is_kept_while_its_arrays_are():
    """Particles.struct: the same ctypes struct for the same fields while the
    container's arrays are the same objects (a load-step-store loop builds it
    once); a replaced array gives a new struct pointing at it; every pointer
    is the array's own, and fields not asked for are null."""
    import numpy as np
    P = abi.Particles(100)
    fin = ("x", "y", "z", "radius", "cell_type")
    s1 = P.struct(fin)
    assert P.struct(fin) is s1
    assert P.struct(("x", "y")) is not s1
    for k in fin:
        assert C.cast(getattr(s1, k), C.c_void_p).value == P[k].ctypes.data, k
    assert not getattr(s1, "velx")
    P["x"] = np.arange(100.0)              # written in place: the same array
    assert P.struct(fin) is s1
    P.a["x"] = np.zeros(100)               # a new array object
    s2 = P.struct(fin)
    assert s2 is not s1
    assert C.cast(s2.x, C.c_void_p).value == P["x"].ctypes.data
    Q = P.copy()                           # a copy has its own arrays and structs
    assert C.cast(Q.struct(fin).x, C.c_void_p).value == Q["x"].ctypes.data
    assert Q.struct(fin).n == P.n
