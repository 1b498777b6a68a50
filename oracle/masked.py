"""Immersed-boundary-masked pressure operator: assembly and direct solve.

Test infrastructure: the oracle of the masked solve.  The reference's
multigrid has no immersed-boundary operator (PLES treats immersed bodies
outside the pressure solve, fsrc/potenziale_ibm.f03:38-87), so this module
restates the reference's discrete system on the fine level -- the 19-point
flux form of resid_sndrcv (fsrc/resid_sndrcv.f03:85-151) and the wall ghost
relation of mul_boun_sndrcv (fsrc/multigrid.f03:1166-1186, homogeneous) with
periodic x and z -- and extends it with a solid-cell mask:

* a face touching a solid cell carries no flux: its normal and both cross
  coefficients are zero;
* a cross coefficient of a fluid-fluid face is zero when its tangential
  stencil reaches a solid cell (wall ghost cells count as the interior cell
  next to them);
* solid cells, and wall ghost cells next to them, are identity rows with a
  zero right-hand side; compatibility and mean refer to the fluid cells.

The singular system is solved exactly (sparse LU) with one interior fluid
equation, implied by the others for a compatible right-hand side, replaced
by a pinned value; the fluid mean is removed afterwards.  With an empty mask the solution
reproduces the converged solution of the restated reference solver
(Oracle.multi); that is how this assembly is pinned.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

# (coefficient, face offset (di,dj,dk) of the coefficient index, sign of the
# flux in the row, [(target offset, weight)]) -- fdx, -fsn, fsop, -fsot, fav,
# -find of resid_sndrcv with the scaled coefficients A = g, B = g/4 (level 1)
_NORMAL = {"a1": ((1, 0, 0), (0, 0, 0)), "a2": ((0, 1, 0), (0, 0, 0)), "a3": ((0, 0, 1), (0, 0, 0))}
_CROSS = {  # face flux cross terms of the face at the low-side cell (i,j,k)
    "b12": [((1, 1, 0), 1), ((0, 1, 0), 1), ((1, -1, 0), -1), ((0, -1, 0), -1)],
    "b13": [((1, 0, 1), 1), ((0, 0, 1), 1), ((1, 0, -1), -1), ((0, 0, -1), -1)],
    "b21": [((1, 1, 0), 1), ((1, 0, 0), 1), ((-1, 1, 0), -1), ((-1, 0, 0), -1)],
    "b23": [((0, 1, 1), 1), ((0, 0, 1), 1), ((0, 1, -1), -1), ((0, 0, -1), -1)],
    "b31": [((1, 0, 1), 1), ((1, 0, 0), 1), ((-1, 0, 1), -1), ((-1, 0, 0), -1)],
    "b32": [((0, 1, 1), 1), ((0, 1, 0), 1), ((0, -1, 1), -1), ((0, -1, 0), -1)],
}
_FACES = {"x": ("a1", "b12", "b13", (1, 0, 0)), "y": ("a2", "b21", "b23", (0, 1, 0)),
          "z": ("a3", "b31", "b32", (0, 0, 1))}


def _coef_boxes(orc, nx, ny, nz):
    """Scaled level-1 coefficients as (nx+2, ny+2, nz+2) arrays indexed by the
    low-side cell of their face, with periodic images in x and z."""
    out = {}
    names = ("g11", "g12", "g13", "g21", "g22", "g23", "g31", "g32", "g33")
    keys = ("a1", "b12", "b13", "b21", "a2", "b23", "b31", "b32", "a3")
    for w, (gname, key) in enumerate(zip(names, keys)):
        g = orc.metric(1, gname)
        box = np.zeros((nx + 2, ny + 2, nz + 2))
        if w < 3:
            box[0:nx + 1, 1:ny + 1, 1:nz + 1] = g
        elif w < 6:
            box[1:nx + 1, 0:ny + 1, 1:nz + 1] = g
        else:
            box[1:nx + 1, 1:ny + 1, 0:nz + 1] = g
        if key[0] == "b":
            box *= 0.25
        # periodic images (faces of ghost cells), as the device boxes hold them
        box[nx + 1, :, :] = box[1, :, :] if w >= 3 else box[nx + 1, :, :]
        box[0, :, :] = box[nx, :, :] if w >= 3 else box[0, :, :]
        if w < 6:
            box[:, :, 0] = box[:, :, nz]
            box[:, :, nz + 1] = box[:, :, 1]
        out[key] = box
    return out


def mask_box(solid, nx, ny, nz):
    """(nx+2, ny+2, nz+2) bool box: periodic images in x/z, wall ghost rows
    copying the interior row next to them."""
    m = np.zeros((nx + 2, ny + 2, nz + 2), dtype=bool)
    s = np.asarray(solid, dtype=bool)
    m[1:nx + 1, 1:ny + 1, 1:nz + 1] = s
    m[1:nx + 1, 0, 1:nz + 1] = s[:, 0, :]
    m[1:nx + 1, ny + 1, 1:nz + 1] = s[:, -1, :]
    m[0] = m[nx]
    m[nx + 1] = m[1]
    m[:, :, 0] = m[:, :, nz]
    m[:, :, nz + 1] = m[:, :, 1]
    return m


def apply_mask(c, m):
    """Zero the coefficients that touch solid cells (rules in the module
    docstring); c: dict of coefficient boxes, m: mask box."""
    nx, ny, nz = (s - 2 for s in m.shape)

    def sh(a, d):  # a[i+di, j+dj, k+dk] for the interior index range used below
        di, dj, dk = d
        return np.roll(a, (-di, -dj, -dk), axis=(0, 1, 2))

    for axis, (an, b1, b2, n) in _FACES.items():
        both = m | sh(m, n)
        t1 = {"x": (0, 1, 0), "y": (1, 0, 0), "z": (1, 0, 0)}[axis]
        t2 = {"x": (0, 0, 1), "y": (0, 0, 1), "z": (0, 1, 0)}[axis]
        def reach(t):
            mt = tuple(-v for v in t)
            n_t = tuple(a + b for a, b in zip(n, t))
            n_mt = tuple(a + b for a, b in zip(n, mt))
            return sh(m, t) | sh(m, mt) | sh(m, n_t) | sh(m, n_mt)
        z1 = reach(t1) & ~both
        z2 = reach(t2) & ~both
        for key in (an, b1, b2):
            c[key][both] = 0.0
        c[b1][z1] = 0.0
        c[b2][z2] = 0.0
    return c


def assemble(c, nx, ny, nz, identity):
    """Sparse matrix of the fine system over unknowns (i=1..nx, j=0..ny+1,
    k=1..nz); identity: bool (nx, ny+2, nz) rows replaced by identity."""
    nj = ny + 2
    n = nx * nz * nj

    def unk(i, j, k):
        return (((k - 1) % nz) * nx + ((i - 1) % nx)) * nj + j

    rows, cols, vals = [], [], []
    I, J, K = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1), np.arange(1, nz + 1), indexing="ij")

    def term(Ir, Jr, Kr, coef, d, w):
        rows.append(unk(Ir, Jr, Kr).ravel())
        cols.append(unk(Ir + d[0], Jr + d[1], Kr + d[2]).ravel())
        vals.append((w * coef).ravel())

    # interior rows: +flux(high face) - flux(low face) for each direction
    for axis, (an, b1, b2, nvec) in _FACES.items():
        for side, sgn in ((0, 1.0), (1, -1.0)):  # high face at the cell, low face at the cell - n
            o = (0, 0, 0) if side == 0 else tuple(-v for v in nvec)
            ci, cj, ck = I + o[0], J + o[1], K + o[2]
            A = c[an][ci, cj, ck]
            hi, lo = _NORMAL[an]
            term(I, J, K, sgn * A, tuple(a + b for a, b in zip(o, hi)), 1.0)
            term(I, J, K, sgn * A, tuple(a + b for a, b in zip(o, lo)), -1.0)
            for bn in (b1, b2):
                B = c[bn][ci, cj, ck]
                for d, w in _CROSS[bn]:
                    term(I, J, K, sgn * B, tuple(a + b for a, b in zip(o, d)), float(w))
    # wall rows (homogeneous): bottom j=0 uses face 0, top j=ny+1 face ny
    I2, K2 = np.meshgrid(np.arange(1, nx + 1), np.arange(1, nz + 1), indexing="ij")
    for jrow, jf, s in ((0, 0, 1.0), (ny + 1, ny, -1.0)):
        J2 = np.full_like(I2, jrow)
        A2, B21, B23 = (c[k][I2, jf, K2] for k in ("a2", "b21", "b23"))
        dn = 1 if jrow == 0 else -1
        term(I2, J2, K2, A2, (0, 0, 0), 1.0)
        term(I2, J2, K2, A2, (0, dn, 0), -1.0)
        # cross terms of the wall face between rows jrow and jrow+dn
        jj = (0, 1) if jrow == 0 else (0, -1)
        for (di, w) in ((1, -s), (-1, s)):
            for dj in jj:
                term(I2, J2, K2, B21, (di, dj, 0), w)
        for (dk, w) in ((1, -s), (-1, s)):
            for dj in jj:
                term(I2, J2, K2, B23, (0, dj, dk), w)
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
    A.sum_duplicates()
    idv = np.zeros(n, dtype=bool)
    Ii, Ji, Ki = np.meshgrid(np.arange(1, nx + 1), np.arange(0, nj), np.arange(1, nz + 1), indexing="ij")
    idv[unk(Ii, Ji, Ki).ravel()] = identity.ravel()
    keep = sp.diags((~idv).astype(float))
    A = keep @ A + sp.diags(idv.astype(float))
    return A.tocsr(), idv, unk


def solve(orc, rhs, solid=None):
    """Converged zero-mean solution (nx, ny, nz) of the masked system for a
    right-hand side (nx, ny, nz); solid (nx, ny, nz) bool or None."""
    nx, ny, nz = orc.dims(1)
    solid = np.zeros((nx, ny, nz), dtype=bool) if solid is None else np.asarray(solid, dtype=bool)
    m = mask_box(solid, nx, ny, nz)
    c = apply_mask(_coef_boxes(orc, nx, ny, nz), m)
    ident = np.zeros((nx, ny + 2, nz), dtype=bool)
    ident[:, 1:ny + 1, :] = solid
    ident[:, 0, :] = solid[:, 0, :]
    ident[:, ny + 1, :] = solid[:, -1, :]
    A, idv, unk = assemble(c, nx, ny, nz, ident)
    n = A.shape[0]
    fluid = ~solid
    b = np.where(fluid, rhs, 0.0)
    b = np.where(fluid, b - b[fluid].mean(), 0.0)
    f = np.zeros(n)
    I, J, K = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1), np.arange(1, nz + 1), indexing="ij")
    qi = unk(I, J, K)
    f[qi.ravel()] = b.ravel()
    # The system is singular (constants on the non-identity unknowns); with a
    # compatible right-hand side one interior fluid equation is implied by the
    # others (the left null vector is +1 on interior rows, -1 on wall rows),
    # so it is replaced by p = 0 at that cell and the fluid mean removed after.
    q0 = int(qi.ravel()[np.flatnonzero(fluid.ravel())[0]])
    A = A.tolil()
    A.rows[q0] = [q0]
    A.data[q0] = [1.0]
    f[q0] = 0.0
    x = spla.spsolve(A.tocsc(), f)
    p = x[qi]
    p = np.where(fluid, p - p[fluid].mean(), 0.0)
    return p


def residual(orc, fi, rhs, solid=None):
    """Masked fine-level residual of a field, vectorised for full-size grids:
    returns (r, rw) with r = L(fi) - b on the interior cells (nx, ny, nz),
    b the fluid-compatible right-hand side of solve() (zero on solid cells,
    where r is zero too), and rw (nx, 2, nz) the residuals of the
    homogeneous wall relations of the bottom (j = 0) and top (j = ny+1)
    ghost rows (zero on rows next to solid cells).  fi (nx+2, ny+2, nz+2)
    holds the field with its ghost layer as a solver returned it; its x/z
    ghost shell is replaced by the periodic images first."""
    nx, ny, nz = orc.dims(1)
    solid = np.zeros((nx, ny, nz), dtype=bool) if solid is None else np.asarray(solid, dtype=bool)
    m = mask_box(solid, nx, ny, nz)
    c = apply_mask(_coef_boxes(orc, nx, ny, nz), m)
    p = np.array(fi, dtype=np.float64, order="F", copy=True)
    p[0] = p[nx]
    p[nx + 1] = p[1]
    p[:, :, 0] = p[:, :, nz]
    p[:, :, nz + 1] = p[:, :, 1]
    I, J, K = slice(1, nx + 1), slice(1, ny + 1), slice(1, nz + 1)

    def P(di, dj, dk, i=I, j=J, k=K):
        return p[i.start + di:i.stop + di, j.start + dj:j.stop + dj, k.start + dk:k.stop + dk]

    def C(key, di, dj, dk):
        return c[key][1 + di:nx + 1 + di, 1 + dj:ny + 1 + dj, 1 + dk:nz + 1 + dk]

    # face fluxes at the high side of each interior cell (o = 0) and the low
    # side (o = -1 along the face normal), the bracketed terms of
    # resid_sndrcv.f03:85-147 with the scaled coefficients
    def fx(o):
        return (C("a1", o, 0, 0) * (P(o + 1, 0, 0) - P(o, 0, 0))
                + C("b12", o, 0, 0) * (P(o + 1, 1, 0) + P(o, 1, 0) - P(o + 1, -1, 0) - P(o, -1, 0))
                + C("b13", o, 0, 0) * (P(o + 1, 0, 1) + P(o, 0, 1) - P(o + 1, 0, -1) - P(o, 0, -1)))

    def fy(o):
        return (C("a2", 0, o, 0) * (P(0, o + 1, 0) - P(0, o, 0))
                + C("b21", 0, o, 0) * (P(1, o + 1, 0) + P(1, o, 0) - P(-1, o + 1, 0) - P(-1, o, 0))
                + C("b23", 0, o, 0) * (P(0, o + 1, 1) + P(0, o, 1) - P(0, o + 1, -1) - P(0, o, -1)))

    def fz(o):
        return (C("a3", 0, 0, o) * (P(0, 0, o + 1) - P(0, 0, o))
                + C("b31", 0, 0, o) * (P(1, 0, o + 1) + P(1, 0, o) - P(-1, 0, o + 1) - P(-1, 0, o))
                + C("b32", 0, 0, o) * (P(0, 1, o + 1) + P(0, 1, o) - P(0, -1, o + 1) - P(0, -1, o)))

    r = fx(0)
    r -= fx(-1)
    r += fy(0)
    r -= fy(-1)
    r += fz(0)
    r -= fz(-1)
    fluid = ~solid
    b = np.where(fluid, rhs, 0.0)
    b = np.where(fluid, b - b[fluid].mean(), 0.0)
    r -= b
    r[solid] = 0.0
    # wall rows: the flux through the wall face (faces 0 and ny) vanishes
    rw = np.zeros((nx, 2, nz))
    for s, (jf, jl) in enumerate(((0, 0), (ny, ny))):
        a2 = c["a2"][I, jf, K]
        b21 = c["b21"][I, jf, K]
        b23 = c["b23"][I, jf, K]

        def Q(di, dj, dk):
            return p[1 + di:nx + 1 + di, jl + dj, 1 + dk:nz + 1 + dk]

        rw[:, s, :] = (a2 * (Q(0, 1, 0) - Q(0, 0, 0)) + b21 * (Q(1, 1, 0) + Q(1, 0, 0) - Q(-1, 1, 0) - Q(-1, 0, 0))
                       + b23 * (Q(0, 1, 1) + Q(0, 0, 1) - Q(0, 1, -1) - Q(0, 0, -1)))
    return r, rw
