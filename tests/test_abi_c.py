"""The C ABI from a compiled C program (tests/abi_check.c): gcc builds it
against include/ples_mg.h and links libples_mg.so, as a non-Python binding
would.  On the CPU it checks the header's struct layout against the layout
the library reports (ples_mg_abi_layout) and that creation reports
PLES_MG_NO_DEVICE; on the GPU it also runs one solve on Fortran-layout
arrays.  The ctypes mirror of ples_gb300.mg is checked against the same
library layout."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

from ples_gb300 import build, mg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lib = build.build()
    exe = str(tmp_path / "abi_check")
    libdir = os.path.dirname(lib)
    cmd = [cc, "-std=c11", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "abi_check.c"), "-o", exe, "-L", libdir, "-lples_mg",
           f"-Wl,-rpath,{libdir}", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_header_layout_matches_the_library(tmp_path):
    exe = _compile(tmp_path)
    r = subprocess.run([exe, "layout"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "FAIL" not in r.stdout
    if not _cuda_available():
        r = subprocess.run([exe, "nodevice"], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr


def test_ctypes_mirror_matches_the_library():
    lib = mg.load()
    v = C.c_int()
    ds, ss = C.c_longlong(), C.c_longlong()
    doff = (C.c_longlong * 24)()
    soff = (C.c_longlong * 8)()
    assert lib.ples_mg_abi_layout(C.byref(v), C.byref(ds), C.byref(ss), doff, soff) == mg.OK
    assert ds.value == C.sizeof(mg.Desc) and ss.value == C.sizeof(mg.Stats)
    assert [getattr(mg.Desc, f).offset for f, _ in mg.Desc._fields_] == list(doff)
    assert [getattr(mg.Stats, f).offset for f, _ in mg.Stats._fields_] == list(soff)


@pytest.mark.gpu
def test_c_caller_solves_on_fortran_layout_arrays(tmp_path):
    exe = _compile(tmp_path)
    r = subprocess.run([exe, "solve"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "rel_residual" in r.stdout
