"""Build the CUDA library libples_mg.so in-tree for GB300 (sm_103a).

Four translation units compiled in parallel with nvcc and linked into one
shared object under ples_gb300/_build/:
  csrc/metric.cu   -- device face metric, compiled with -fmad=false so its
                      FP64 arithmetic is rounded as written
  csrc/ples_mg.cu  -- stencil kernels, V-cycle driver and the C ABI
  csrc/batch.cu    -- batched solves of many grids and the request server
  csrc/grid_io.cpp -- reader of PLES's grid file (host code)
The library depends on the CUDA runtime only (statically linked; NVTX ranges
come from the toolkit's header-only NVTX v3); PyTorch is not needed to build
or load it.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libples_mg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libples_mg.so")


def _sources():
    return [os.path.join(SRC, f) for f in sorted(os.listdir(SRC))] + [
        os.path.join(ROOT, "include", "ples_mg.h")]


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(s) > t for s in _sources())


def build(force=False, verbose=False, extra=()):
    """Compile and link; returns the library path."""
    if not force and not needs_build():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = nvcc_path()
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", SRC,
              "-I", os.path.join(ROOT, "include")] + ARCH + list(extra)
    units = [("metric.cu", ["-fmad=false"]), ("ples_mg.cu", []), ("batch.cu", []), ("grid_io.cpp", [])]
    procs = []
    for name, flags in units:
        obj = os.path.join(OUT, os.path.splitext(name)[0] + ".o")
        cmd = [nvcc] + common + flags + ["-c", os.path.join(SRC, name), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((name, obj, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    objs = []
    for name, obj, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed on {name}:\n{out.decode(errors='replace')}")
        if verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
        objs.append(obj)
    tmp = LIB + ".tmp"
    cmd = [nvcc, "-shared"] + ARCH + ["-o", tmp] + objs + ["-lpthread", "-ldl"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout.decode(errors='replace')}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
