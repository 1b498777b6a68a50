"""Host-side interface of the GB300 pressure multigrid, over the C ABI.

`Multigrid` mirrors the reference's set-up/solve split: construction plays
the part of metrica -> mul_met -> wall (fsrc/stratiParticle.f03:767-769) and
`multi(eps, ficycle, fi, rhs)` keeps the meaning of the Fortran subroutine
`multi` (fsrc/multigrid.f03:42-653): an absolute max-norm stop `eps`, at most
`ficycle` cycles, `fi` updated in place including its ghost layer.  `solve`
adds the relative L2 stop used by the benchmarks.

Everything runs in libples_mg.so on the GPU; if the library cannot be built
or loaded, or no GPU is present, construction raises -- there is no CPU path.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

OK, NOT_CONVERGED, BAD_ARG, OOM, DEVICE_TIMEOUT, CUDA_ERROR, DIVERGED, NO_DEVICE = range(8)
PREC_FP64, PREC_MIXED, PREC_OUTER = 0, 1, 2
COORDS_NODES, COORDS_GHOSTED8 = 0, 1
METRIC_NAMES = ("g11", "g12", "g13", "g21", "g22", "g23", "g31", "g32", "g33")


class PlesMGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class Desc(C.Structure):
    _fields_ = [("jx", C.c_int), ("jy", C.c_int), ("jz", C.c_int),
                ("ip", C.c_int), ("jp", C.c_int), ("kp", C.c_int),
                ("nlevmax", C.c_int), ("omega", C.c_double), ("precision", C.c_int),
                ("coords_layout", C.c_int),
                ("x", C.POINTER(C.c_double)), ("y", C.POINTER(C.c_double)),
                ("z", C.POINTER(C.c_double)), ("dt", C.c_double), ("device", C.c_int),
                ("nu_pre", C.c_int), ("nu_post", C.c_int), ("nu_coarse", C.c_int),
                ("inner_cycles", C.c_int), ("smoother", C.c_int), ("coarsening", C.c_int),
                ("solid", C.c_void_p), ("tipo", C.c_void_p), ("freesurface", C.c_int)]


class Tuning(C.Structure):
    _fields_ = [("nu", C.c_int), ("inner_cycles", C.c_int), ("line_threads", C.c_int * 12),
                ("solve_ms", C.c_double), ("candidates", C.c_int), ("nu_post", C.c_int), ("omega", C.c_double)]


class Stats(C.Structure):
    _fields_ = [("outer_iterations", C.c_int), ("vcycles", C.c_int),
                ("rel_residual", C.c_double), ("max_residual", C.c_double),
                ("rhs_norm", C.c_double), ("rhs_mean_removed", C.c_double),
                ("seconds", C.c_double), ("status", C.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="F_CONTIGUOUS")

EXPORTS = ("ples_mg_create", "ples_mg_solve", "ples_mg_solve_device", "ples_mg_destroy",
           "ples_mg_strerror", "ples_mg_last_error", "ples_mg_levels", "ples_mg_level_dims",
           "ples_mg_get_metric", "ples_mg_apply_residual", "ples_mg_apply_ghost_fill",
           "ples_mg_apply_restrict", "ples_mg_apply_prolong", "ples_mg_counters",
           "ples_mg_kernel_timing", "ples_mg_kernel_time", "ples_mg_batch_create",
           "ples_mg_batch_solve", "ples_mg_batch_solve_device", "ples_mg_batch_info",
           "ples_mg_batch_last_error", "ples_mg_batch_destroy", "ples_srv_create", "ples_srv_submit",
           "ples_srv_wait", "ples_srv_report", "ples_srv_destroy", "ples_mg_autotune", "ples_mg_project",
           "ples_mg_step", "ples_mg_residual_norms_device", "ples_mg_read_grid", "ples_mg_potenziale_ibm",
           "ples_mg_set_line_threads", "ples_mg_get_line_threads", "ples_mg_set_surface_pressure",
           "ples_mg_abi_layout", "ples_mg_set_wait_limit")
KERNEL_KINDS = {"line": 0, "restrict": 1, "prolong": 2, "outer": 3}


def load(build=True):
    """Load libples_mg.so (building it first if its sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build else _build.LIB
    if not os.path.exists(path):
        raise ImportError(f"libples_mg.so not found at {path}; run ples_gb300/build.py")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.ples_mg_create.argtypes = [C.POINTER(Desc), C.POINTER(vp)]
    L.ples_mg_solve.argtypes = [vp, _dp, _dp, vp, C.c_double, C.c_double, C.c_int, C.POINTER(Stats)]
    L.ples_mg_solve_device.argtypes = [vp, vp, vp, vp, C.c_double, C.c_double, C.c_int, vp,
                                       C.POINTER(Stats)]
    L.ples_mg_destroy.argtypes = [vp]
    L.ples_mg_destroy.restype = None
    L.ples_mg_strerror.restype = C.c_char_p
    L.ples_mg_strerror.argtypes = [C.c_int]
    L.ples_mg_last_error.restype = C.c_char_p
    L.ples_mg_last_error.argtypes = [vp]
    L.ples_mg_levels.argtypes = [vp, C.POINTER(C.c_int)]
    L.ples_mg_level_dims.argtypes = [vp, C.c_int] + [C.POINTER(C.c_int)] * 3
    L.ples_mg_get_metric.argtypes = [vp, C.c_int, C.c_int, _dp]
    L.ples_mg_apply_residual.argtypes = [vp, C.c_int, _dp, _dp, _dp, C.c_int]
    L.ples_mg_apply_ghost_fill.argtypes = [vp, C.c_int, _dp, vp, C.c_int]
    L.ples_mg_apply_restrict.argtypes = [vp, C.c_int, _dp, _dp]
    L.ples_mg_apply_prolong.argtypes = [vp, C.c_int, _dp, _dp]
    L.ples_mg_counters.argtypes = [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
    L.ples_mg_kernel_timing.argtypes = [vp, C.c_int, C.c_int]
    L.ples_mg_kernel_time.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
    L.ples_mg_residual_norms_device.argtypes = [vp, vp, vp, vp, vp, C.POINTER(C.c_double)]
    L.ples_mg_autotune.argtypes = [vp, vp, C.POINTER(Tuning)]
    L.ples_mg_set_line_threads.argtypes = [vp, C.c_int, C.c_int]
    L.ples_mg_get_line_threads.argtypes = [vp, C.c_int, C.POINTER(C.c_int)]
    L.ples_mg_set_surface_pressure.argtypes = [vp, vp]
    L.ples_mg_set_wait_limit.argtypes = [vp, C.c_longlong]
    LL = C.POINTER(C.c_longlong)
    L.ples_mg_abi_layout.argtypes = [C.POINTER(C.c_int), LL, LL, LL, LL]
    L.ples_mg_project.argtypes = [vp] + [vp] * 7 + [C.c_double, C.c_int, C.POINTER(Stats)]
    L.ples_mg_step.argtypes = [vp] + [vp] * 7 + [C.c_double, C.c_int, C.POINTER(Stats)]
    L.ples_mg_read_grid.argtypes = [C.c_char_p, vp, vp, vp, vp, vp]
    L.ples_mg_potenziale_ibm.argtypes = [vp, vp]
    L.ples_mg_batch_create.argtypes = [vp, C.c_int, C.POINTER(vp)]
    L.ples_mg_batch_solve.argtypes = [vp, vp, vp, C.c_double, C.c_int, vp]
    L.ples_mg_batch_solve_device.argtypes = [vp, vp, vp, C.c_double, C.c_int, vp]
    L.ples_mg_batch_info.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_longlong)]
    L.ples_mg_batch_last_error.argtypes = [vp]
    L.ples_mg_batch_last_error.restype = C.c_char_p
    L.ples_mg_batch_destroy.argtypes = [vp]
    L.ples_mg_batch_destroy.restype = None
    L.ples_srv_create.argtypes = [vp, C.c_int, C.c_double, C.POINTER(vp)]
    L.ples_srv_submit.argtypes = [vp, C.c_int, vp, vp, C.c_double, C.c_int, C.POINTER(C.c_longlong)]
    L.ples_srv_wait.argtypes = [vp, C.c_longlong, C.POINTER(Stats)]
    L.ples_srv_report.argtypes = [vp] + [C.POINTER(C.c_double)] * 3 + [C.POINTER(C.c_longlong),
                                                                       C.POINTER(C.c_double)]
    L.ples_srv_destroy.argtypes = [vp]
    L.ples_srv_destroy.restype = None
    _lib = L
    return L


def _f64(a):
    return np.asfortranarray(a, dtype=np.float64)


def _cs_ptrs(cs):
    if cs is None:
        return None, None
    keep = [None if a is None else _f64(a) for a in cs]
    arr = (C.c_void_p * 6)(*[None if a is None else a.ctypes.data for a in keep])
    return C.cast(arr, C.c_void_p), (keep, arr)


def read_grid(path):
    """PLES's grid file through ples_mg_read_grid: returns (lengths, (jx, jy,
    jz), (x, y, z)) with node arrays (jx+1, jy+1, jz+1) in Fortran order."""
    L = load()
    lengths = (C.c_double * 3)()
    dims = (C.c_int * 3)()
    rc = L.ples_mg_read_grid(os.fsencode(path), lengths, dims, None, None, None)
    if rc:
        raise PlesMGError(rc, f"{L.ples_mg_strerror(rc).decode()}: cannot read grid file {path}")
    jx, jy, jz = dims
    xyz = [np.zeros((jx + 1, jy + 1, jz + 1), order="F") for _ in range(3)]
    rc = L.ples_mg_read_grid(os.fsencode(path), lengths, dims, *[C.c_void_p(a.ctypes.data) for a in xyz])
    if rc:
        raise PlesMGError(rc, f"{L.ples_mg_strerror(rc).decode()}: malformed grid file {path}")
    return tuple(lengths), (jx, jy, jz), tuple(xyz)


class Multigrid:
    """One grid's coefficient hierarchy, resident on the GPU."""

    def __init__(self, x, y, z, ip=0, jp=1, kp=0, precision="mixed", dt=1.0, device=0,
                 nlevmax=0, omega=0.0, nu_pre=0, nu_post=0, nu_coarse=0, inner_cycles=0,
                 smoother=0, coarsening=0, coords_layout=COORDS_NODES, solid=None, tipo=None,
                 freesurface=0):
        self._L = load()
        self._x, self._y, self._z = _f64(x), _f64(y), _f64(z)
        if coords_layout == COORDS_NODES:
            jx, jy, jz = (s - 1 for s in self._x.shape)
        else:
            jx, jy, jz = (s - 17 for s in self._x.shape)
        self.jx, self.jy, self.jz = jx, jy, jz
        self.precision = {"mixed": PREC_MIXED, "fp64": PREC_FP64}.get(precision, precision)
        d = Desc()
        d.jx, d.jy, d.jz, d.ip, d.jp, d.kp = jx, jy, jz, ip, jp, kp
        d.nlevmax, d.omega, d.precision, d.coords_layout = nlevmax, omega, self.precision, coords_layout
        dp = C.POINTER(C.c_double)
        d.x = self._x.ctypes.data_as(dp)
        d.y = self._y.ctypes.data_as(dp)
        d.z = self._z.ctypes.data_as(dp)
        d.dt, d.device = dt, device
        d.nu_pre, d.nu_post, d.nu_coarse = nu_pre, nu_post, nu_coarse
        d.inner_cycles, d.smoother, d.coarsening = inner_cycles, smoother, coarsening
        d.freesurface = freesurface
        self._solid = None
        if solid is not None:  # immersed-boundary mask (jx, jy, jz), nonzero = solid
            self._solid = np.asfortranarray(np.asarray(solid) != 0, dtype=np.uint8)
            if self._solid.shape != (jx, jy, jz):
                raise ValueError(f"solid mask must be {(jx, jy, jz)}")
            d.solid = self._solid.ctypes.data
        self._tipo = None
        if tipo is not None:  # PLES cell types (jx+2, jy+2, jz+2): 0 solid, 1 IB, >= 2 fluid
            self._tipo = np.asfortranarray(tipo, dtype=np.int32)
            if self._tipo.shape != (jx + 2, jy + 2, jz + 2):
                raise ValueError(f"tipo must be {(jx + 2, jy + 2, jz + 2)}")
            d.tipo = self._tipo.ctypes.data
        h = C.c_void_p()
        rc = self._L.ples_mg_create(C.byref(d), C.byref(h))
        if rc != OK:
            raise PlesMGError(rc, self._L.ples_mg_strerror(rc).decode())
        self._h = h

    # -- lifetime --------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._L.ples_mg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc, allow=(OK,)):
        if rc not in allow:
            msg = self._L.ples_mg_last_error(self._h).decode() if self._h else ""
            raise PlesMGError(rc, f"{self._L.ples_mg_strerror(rc).decode()}: {msg}")
        return rc

    # -- levels ------------------------------------------------------------
    @property
    def nlevel(self):
        n = C.c_int()
        self._check(self._L.ples_mg_levels(self._h, C.byref(n)))
        return n.value

    def dims(self, level):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        self._check(self._L.ples_mg_level_dims(self._h, level, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    # -- solves --------------------------------------------------------------
    def solve(self, rhs, fi=None, cs=None, rel_tol=1e-10, abs_tol=0.0, max_cycles=200):
        """Returns (fi, stats dict); fi (jx+2, jy+2, jz+2) with ghosts."""
        if fi is None:
            fi = np.zeros((self.jx + 2, self.jy + 2, self.jz + 2), order="F")
        else:
            fi = _f64(fi).copy(order="F")
        st = Stats()
        ptr, keep = _cs_ptrs(cs)
        rc = self._L.ples_mg_solve(self._h, fi, _f64(rhs), ptr, rel_tol, abs_tol, max_cycles,
                                   C.byref(st))
        self._check(rc, allow=(OK, NOT_CONVERGED))
        return fi, st.as_dict()

    def multi(self, eps, ficycle, fi, rhs, cs=None):
        """The reference's entry point: fi updated in place, stop on
        max|r| < eps or ficycle cycles; returns the cycle count."""
        if not (isinstance(fi, np.ndarray) and fi.dtype == np.float64 and fi.flags.f_contiguous):
            raise TypeError("fi must be a Fortran-ordered float64 array (0:jx+1,0:jy+1,0:jz+1)")
        st = Stats()
        ptr, keep = _cs_ptrs(cs)
        rc = self._L.ples_mg_solve(self._h, fi, _f64(rhs), ptr, 0.0, eps, ficycle, C.byref(st))
        self._check(rc, allow=(OK, NOT_CONVERGED))
        return st.outer_iterations

    def solve_device(self, d_fi, d_rhs, rel_tol=1e-10, abs_tol=0.0, max_cycles=200, stream=0,
                     d_cs=None):
        """Device-resident solve; d_fi/d_rhs are CUDA buffers (integer device
        pointers, e.g. torch_tensor.data_ptr()) in Fortran layout."""
        st = Stats()
        ptr = None
        if d_cs is not None:
            arr = (C.c_void_p * 6)(*[None if p is None else int(p) for p in d_cs])
            ptr = C.cast(arr, C.c_void_p)
        rc = self._L.ples_mg_solve_device(self._h, C.c_void_p(int(d_fi)), C.c_void_p(int(d_rhs)), ptr,
                                          rel_tol, abs_tol, max_cycles, C.c_void_p(int(stream)),
                                          C.byref(st))
        self._check(rc, allow=(OK, NOT_CONVERGED))
        return st.as_dict()

    def residual_norms_device(self, d_fi, d_rhs, d_r=0, stream=0):
        """Fine-level r = L(fi) - rhs from device buffers (integer device
        pointers, Fortran layout) without any device allocation; returns
        (sum of r^2, max |r|) and writes r to d_r unless it is 0."""
        out = (C.c_double * 2)()
        self._check(self._L.ples_mg_residual_norms_device(
            self._h, C.c_void_p(int(d_fi)), C.c_void_p(int(d_rhs)), C.c_void_p(int(d_r) or None),
            C.c_void_p(int(stream) or None), out))
        return out[0], out[1]

    def project(self, uc, vc, wc, fi, u=None, v=None, w=None, rel_tol=1e-10, max_cycles=200):
        """Projection step (diver, solve, gradie, vel_up): returns the new
        (uc, vc, wc, fi) and, if given, (u, v, w); inputs are not modified."""
        jx, jy, jz = self.jx, self.jy, self.jz
        shapes = [(jx + 1, jy, jz), (jx, jy + 1, jz), (jx, jy, jz + 1)] + [(jx + 2, jy + 2, jz + 2)] * 4
        arrs = [None if a is None else _f64(a).copy(order="F") for a in (uc, vc, wc, fi, u, v, w)]
        for a, sh in zip(arrs, shapes):
            if a is not None and a.shape != sh:
                raise ValueError(f"array of shape {a.shape}, expected {sh}")
        ptr = [None if a is None else C.c_void_p(a.ctypes.data) for a in arrs]
        st = Stats()
        rc = self._L.ples_mg_project(self._h, ptr[0], ptr[1], ptr[2], ptr[4], ptr[5], ptr[6], ptr[3], rel_tol,
                                     max_cycles, C.byref(st))
        self._check(rc, allow=(OK, NOT_CONVERGED))
        out = arrs[:4] + ([arrs[4], arrs[5], arrs[6]] if u is not None else [])
        return out, st.as_dict()

    def potenziale_ibm(self, fi):
        """Solid cells (tipo 0) of fi take the mean of their IB neighbours
        (ples_mg_potenziale_ibm); returns a new array."""
        a = _f64(fi).copy(order="F")
        if a.shape != (self.jx + 2, self.jy + 2, self.jz + 2):
            raise ValueError(f"fi of shape {a.shape}")
        self._check(self._L.ples_mg_potenziale_ibm(self._h, C.c_void_p(a.ctypes.data)))
        return a

    def step(self, u, v, w, uc, vc, wc, fi, rel_tol=1e-10, max_cycles=200):
        """The pressure step from the intermediate Cartesian velocities
        (contra, diver, solve, gradie, vel_up): returns the new
        (u, v, w, uc, vc, wc, fi); inputs are not modified."""
        jx, jy, jz = self.jx, self.jy, self.jz
        cell = (jx + 2, jy + 2, jz + 2)
        shapes = [cell] * 3 + [(jx + 1, jy, jz), (jx, jy + 1, jz), (jx, jy, jz + 1), cell]
        arrs = [_f64(a).copy(order="F") for a in (u, v, w, uc, vc, wc, fi)]
        for a, sh in zip(arrs, shapes):
            if a.shape != sh:
                raise ValueError(f"array of shape {a.shape}, expected {sh}")
        st = Stats()
        rc = self._L.ples_mg_step(self._h, *[C.c_void_p(a.ctypes.data) for a in arrs], rel_tol, max_cycles,
                                  C.byref(st))
        self._check(rc, allow=(OK, NOT_CONVERGED))
        return arrs, st.as_dict()

    def autotune(self, rhs=None):
        """Time candidate smoother widths, sweep counts (before / after the
        coarse correction), inner cycles and omega on this grid and keep the
        fastest (ples_mg_autotune)."""
        t = Tuning()
        keep = None if rhs is None else _f64(rhs)
        ptr = None if keep is None else C.c_void_p(keep.ctypes.data)
        self._check(self._L.ples_mg_autotune(self._h, ptr, C.byref(t)))
        return {"nu": t.nu, "nu_pre": t.nu, "nu_post": t.nu_post, "omega": t.omega, "inner_cycles": t.inner_cycles,
                "line_threads": [v for v in t.line_threads if v], "solve_ms": t.solve_ms,
                "candidates": t.candidates}

    def set_line_threads(self, level, threads):
        """Smoother form at one level (1-based): 128, 256 or 512 threads on
        32-line tiles, 1024 for the 64-line tiles, 2048 for the same tiles
        with rows built two lines per thread, 4096 for the 64-line tiles
        with both k parities in one launch (ples_mg_set_line_threads)."""
        self._check(self._L.ples_mg_set_line_threads(self._h, level, threads))

    def set_surface_pressure(self, next_prs=None):
        """Surface pressure PrS0 (jx, jz) of a free-surface handle for the
        following solves (ples_mg_set_surface_pressure); None = zero."""
        ptr = None
        if next_prs is not None:
            self._prs = _f64(next_prs)
            if self._prs.shape != (self.jx, self.jz):
                raise ValueError(f"next_prs must be {(self.jx, self.jz)}")
            ptr = self._prs.ctypes.data
        self._check(self._L.ples_mg_set_surface_pressure(self._h, ptr))

    def set_wait_limit(self, polls=-1):
        """Polls of a bounded device wait before it gives up (-1: default)."""
        self._check(self._L.ples_mg_set_wait_limit(self._h, polls))

    def line_threads(self, level):
        """The smoother form at one level (ples_mg_get_line_threads)."""
        t = C.c_int()
        self._check(self._L.ples_mg_get_line_threads(self._h, level, C.byref(t)))
        return t.value

    # -- instrumentation ------------------------------------------------------
    def counters(self):
        n, b = C.c_longlong(), C.c_longlong()
        self._check(self._L.ples_mg_counters(self._h, C.byref(n), C.byref(b)))
        return {"launches": n.value, "device_bytes": b.value}

    def time_kernel(self, kind, level=1):
        """Start CUDA-event timing of one kernel kind ('line', 'restrict',
        'prolong', 'outer' or None to stop) at one level."""
        k = -1 if kind is None else KERNEL_KINDS[kind]
        self._check(self._L.ples_mg_kernel_timing(self._h, k, level))

    def kernel_time(self):
        ms, n = C.c_double(), C.c_longlong()
        self._check(self._L.ples_mg_kernel_time(self._h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    # -- per-level operators -------------------------------------------------
    def metric(self, level, which):
        w = METRIC_NAMES.index(which)
        nx, ny, nz = self.dims(level)
        shape = [(nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1)][w // 3]
        out = np.zeros(shape, order="F")
        self._check(self._L.ples_mg_get_metric(self._h, level, w, out))
        return out

    def residual(self, level, pr, rh, precision="fp64"):
        """L(pr) - rh at one level (ples_mg_apply_residual): the FP64 kernel,
        the FP32 one ("fp32"), or ("outer", level 1) the one the solve's stop
        test uses: double-float products on a mixed handle."""
        nx, ny, nz = self.dims(level)
        out = np.zeros((nx, ny, nz), order="F")
        p = {"fp64": PREC_FP64, "fp32": PREC_MIXED, "mixed": PREC_MIXED, "outer": PREC_OUTER}[precision]
        self._check(self._L.ples_mg_apply_residual(self._h, level, _f64(pr), _f64(rh), out, p))
        return out

    def ghost_fill(self, level, pr, cs=None, passes=30):
        pr = _f64(pr).copy(order="F")
        ptr, keep = _cs_ptrs(cs)
        self._check(self._L.ples_mg_apply_ghost_fill(self._h, level, pr, ptr, passes))
        return pr

    def restrict(self, level, rh):
        nx, ny, nz = self.dims(level + 1)
        out = np.zeros((nx, ny, nz), order="F")
        self._check(self._L.ples_mg_apply_restrict(self._h, level, _f64(rh), out))
        return out

    def prolong(self, level, prf, prc):
        prf = _f64(prf).copy(order="F")
        self._check(self._L.ples_mg_apply_prolong(self._h, level, prf, _f64(prc)))
        return prf


def _ptr_array(ptrs):
    arr = (C.c_void_p * len(ptrs))(*[None if p is None else int(p) for p in ptrs])
    return arr


class Batch:
    """Many grids solved together (ples_mg_batch_*): the members are
    Multigrid objects that keep their resident hierarchies.  Mixed-precision
    members with the zebra smoother, full coarsening, periodic x and z and a
    dense coarsest level share the batched step list; any other member is
    solved by the single-grid solver within the same call."""

    def __init__(self, members):
        self._L = load()
        self.members = list(members)
        hs = (C.c_void_p * len(self.members))(*[m._h.value for m in self.members])
        b = C.c_void_p()
        rc = self._L.ples_mg_batch_create(C.cast(hs, C.c_void_p), len(self.members), C.byref(b))
        if rc != OK:
            raise PlesMGError(rc, self._L.ples_mg_strerror(rc).decode())
        self._b = b

    def close(self):
        if getattr(self, "_b", None):
            self._L.ples_mg_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc, allow=(OK, NOT_CONVERGED)):
        if rc not in allow:
            raise PlesMGError(rc, f"{self._L.ples_mg_strerror(rc).decode()}: "
                                  f"{self._L.ples_mg_batch_last_error(self._b).decode()}")
        return rc

    def solve(self, rhs_list, fi_list=None, rel_tol=1e-10, max_cycles=200):
        """Host arrays; returns (list of fi, list of stats dicts).  fi_list
        None starts every member from zero."""
        n = len(self.members)
        if fi_list is None:
            fi_list = [np.zeros((m.jx + 2, m.jy + 2, m.jz + 2), order="F") for m in self.members]
        fis = [_f64(f).copy(order="F") for f in fi_list]
        rhs = [_f64(r) for r in rhs_list]
        for m, f, r in zip(self.members, fis, rhs, strict=True):
            if f.shape != (m.jx + 2, m.jy + 2, m.jz + 2) or r.shape != (m.jx, m.jy, m.jz):
                raise ValueError("fi/rhs shapes must match the members' grids")
        st = (Stats * n)()
        rc = self._L.ples_mg_batch_solve(self._b, C.cast(_ptr_array([f.ctypes.data for f in fis]), C.c_void_p),
                                         C.cast(_ptr_array([r.ctypes.data for r in rhs]), C.c_void_p),
                                         rel_tol, max_cycles, C.cast(st, C.c_void_p))
        self._check(rc)
        return fis, [s.as_dict() for s in st]

    def solve_device(self, d_fi, d_rhs, rel_tol=1e-10, max_cycles=200):
        """Device buffers (integer pointers) in the Fortran layouts."""
        n = len(self.members)
        st = (Stats * n)()
        rc = self._L.ples_mg_batch_solve_device(self._b, C.cast(_ptr_array(d_fi), C.c_void_p),
                                                C.cast(_ptr_array(d_rhs), C.c_void_p), rel_tol, max_cycles,
                                                C.cast(st, C.c_void_p))
        self._check(rc)
        return [s.as_dict() for s in st]

    def info(self):
        s, r = C.c_int(), C.c_longlong()
        self._L.ples_mg_batch_info(self._b, C.byref(s), C.byref(r))
        return {"steps": s.value, "replays": r.value}


class Server:
    """Request server with continuous batching (ples_srv_*)."""

    def __init__(self, members, hbm_budget_bytes=0.0):
        self._L = load()
        self.members = list(members)
        hs = (C.c_void_p * len(self.members))(*[m._h.value for m in self.members])
        s = C.c_void_p()
        rc = self._L.ples_srv_create(C.cast(hs, C.c_void_p), len(self.members), hbm_budget_bytes, C.byref(s))
        if rc != OK:
            raise PlesMGError(rc, self._L.ples_mg_strerror(rc).decode())
        self._s = s
        self._out = {}

    def close(self):
        if getattr(self, "_s", None):
            self._L.ples_srv_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, member, rhs, rel_tol=1e-10, max_cycles=200):
        m = self.members[member]
        out = np.zeros((m.jx + 2, m.jy + 2, m.jz + 2), order="F")
        r = _f64(rhs)  # held until the call returns: the server copies it
        if r.shape != (m.jx, m.jy, m.jz):
            raise ValueError(f"rhs of member {member} must be {(m.jx, m.jy, m.jz)}")
        t = C.c_longlong()
        rc = self._L.ples_srv_submit(self._s, member, C.c_void_p(r.ctypes.data),
                                     C.c_void_p(out.ctypes.data), rel_tol, max_cycles, C.byref(t))
        if rc != OK:
            raise PlesMGError(rc, self._L.ples_mg_strerror(rc).decode())
        self._out[t.value] = out
        return t.value

    def wait(self, ticket):
        """Returns (fi, stats dict); stats['seconds'] is the request latency."""
        st = Stats()
        rc = self._L.ples_srv_wait(self._s, ticket, C.byref(st))
        out = self._out.pop(ticket, None)
        if rc not in (OK, NOT_CONVERGED):
            raise PlesMGError(rc, self._L.ples_mg_strerror(rc).decode())
        return out, st.as_dict()

    def report(self):
        a, b, c, sps = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        n = C.c_longlong()
        self._L.ples_srv_report(self._s, C.byref(a), C.byref(b), C.byref(c), C.byref(n), C.byref(sps))
        return {"p50_ms": a.value, "p99_ms": b.value, "p999_ms": c.value, "completed": n.value,
                "solves_per_s": sps.value}
