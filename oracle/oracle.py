"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests, the smoke check and the CPU-baseline leg of the benchmark use
this module.  It loads oracle/_build/libples_oracle.so (built by
``make -C oracle``) and exposes the restated PLES multigrid routines on
numpy arrays in Fortran order with the reference's extents.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libples_oracle.so")
_lib = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="F_CONTIGUOUS")


def build(force=False):
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "ples_oracle.c"))
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.c_int] * 8 + [C.c_double, C.c_int, C.c_double, _dp, _dp, _dp]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_last_error.restype = C.c_char_p
        L.orc_nlevel.argtypes = [C.c_void_p]
        L.orc_level_dims.argtypes = [C.c_void_p, C.c_int] + [C.POINTER(C.c_int)] * 3
        L.orc_get_metric.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp]
        L.orc_get_coords.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_resid.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp]
        L.orc_ghost_fill.argtypes = [C.c_void_p, C.c_int, _dp, C.c_void_p]
        L.orc_restrict.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
        L.orc_prolong.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
        L.orc_multi.argtypes = [C.c_void_p, _dp, _dp, C.c_void_p, C.c_double, C.c_int, C.c_int,
                                C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_true_residual.argtypes = [C.c_void_p, _dp, _dp, C.c_void_p, _dp, C.c_int]
        L.orc_set_free_surface.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        _lib = L
    return _lib


def _f(a):
    return np.asfortranarray(a, dtype=np.float64)


class Oracle:
    """One restated PLES multigrid problem (grid, metric hierarchy, masks)."""

    def __init__(self, x, y, z, ip=0, jp=1, kp=0, nlevmax=4, nproc=1, omega=1.6,
                 islor=0, dt=1.0):
        L = lib()
        jx, jy, jz = (s - 1 for s in x.shape)
        self.jx, self.jy, self.jz = jx, jy, jz
        self.ip, self.jp, self.kp, self.dt = ip, jp, kp, dt
        self._x, self._y, self._z = _f(x), _f(y), _f(z)
        h = L.orc_create(jx, jy, jz, ip, jp, kp, nlevmax, nproc, omega, islor, dt,
                         self._x, self._y, self._z)
        if not h:
            raise ValueError(L.orc_last_error().decode())
        self._h = h
        self.nlevel = L.orc_nlevel(h)

    def close(self):
        if self._h:
            lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_free_surface(self, on=True, next_prs=None):
        """multi's freesurface argument and the surface pressure next_prs
        (jx, jz) of level 1 (None: the first time step, PrS0 = 0)."""
        self._prs = None if next_prs is None else _f(next_prs)
        if self._prs is not None and self._prs.shape != (self.jx, self.jz):
            raise ValueError("next_prs must be (jx, jz)")
        ptr = None if self._prs is None else self._prs.ctypes.data
        if lib().orc_set_free_surface(self._h, 1 if on else 0, ptr):
            raise ValueError("bad free-surface setting")

    def dims(self, n):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        lib().orc_level_dims(self._h, n, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value

    def metric(self, n, which):
        """which: 'g11'..'g33' or 'giac'; arrays with the reference extents."""
        names = ["g11", "g12", "g13", "g21", "g22", "g23", "g31", "g32", "g33", "giac"]
        w = names.index(which)
        nx, ny, nz = self.dims(n)
        shape = {0: (nx + 1, ny, nz), 1: (nx, ny + 1, nz), 2: (nx, ny, nz + 1), 3: (nx, ny, nz)}[
            3 if w == 9 else w // 3]
        out = np.zeros(shape, order="F")
        if lib().orc_get_metric(self._h, n, w, out):
            raise ValueError("bad level/metric")
        return out

    def coords(self, c):
        out = np.zeros((self.jx + 17, self.jy + 17, self.jz + 17), order="F")
        lib().orc_get_coords(self._h, c, out)
        return out

    @staticmethod
    def _cs(cs):
        if cs is None:
            return None, None
        keep = [None if a is None else _f(a) for a in cs]
        arr = (C.c_void_p * 6)(*[None if a is None else a.ctypes.data for a in keep])
        return C.cast(arr, C.c_void_p), (keep, arr)

    def resid(self, n, pr, rh):
        nx, ny, nz = self.dims(n)
        out = np.zeros((nx, ny, nz), order="F")
        lib().orc_resid(self._h, n, _f(pr), _f(rh), out)
        return out

    def ghost_fill(self, n, pr, cs=None):
        pr = _f(pr).copy(order="F")
        ptr, keep = self._cs(cs)
        lib().orc_ghost_fill(self._h, n, pr, ptr)
        return pr

    def restrict(self, n, rh):
        nx, ny, nz = self.dims(n + 1)
        out = np.zeros((nx, ny, nz), order="F")
        lib().orc_restrict(self._h, n, _f(rh), out)
        return out

    def prolong(self, n, prf, prc):
        prf = _f(prf).copy(order="F")
        lib().orc_prolong(self._h, n, prf, _f(prc))
        return prf

    def multi(self, rhs, fi=None, cs=None, eps=1e-10, ficycle=1000, stop_mode=1):
        """Run the V-cycle driver; returns (fi, cycles, max|r|, ||r||/||b||)."""
        if fi is None:
            fi = np.zeros((self.jx + 2, self.jy + 2, self.jz + 2), order="F")
        fi = _f(fi).copy(order="F")
        ptr, keep = self._cs(cs)
        cyc, rm, rr = C.c_int(), C.c_double(), C.c_double()
        rc = lib().orc_multi(self._h, fi, _f(rhs), ptr, eps, ficycle, stop_mode,
                             C.byref(cyc), C.byref(rm), C.byref(rr))
        if rc:
            raise ValueError(lib().orc_last_error().decode())
        return fi, cyc.value, rm.value, rr.value

    def true_residual(self, fi, rhs, cs=None, passes=20):
        fi = _f(fi).copy(order="F")
        out = np.zeros((self.jx, self.jy, self.jz), order="F")
        ptr, keep = self._cs(cs)
        lib().orc_true_residual(self._h, fi, _f(rhs), ptr, out, passes)
        return out, fi
