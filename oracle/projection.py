"""Projection step either side of the pressure solve: diver, gradie, vel_up.

Test infrastructure: the oracle of ples_mg_project and ples_mg_step.
Restates, for a single domain with periodic x and z and walls in y
(ip = kp = 0, jp = 1), potenziale = 0 and no free surface:

* contra (fsrc/contra.f03:91-219): uc, vc, wc from the Cartesian u, v, w
  averaged onto the faces, and the wall fluxes cs3, cs4 (new minus old vc
  on the wall faces);
* diver  (fsrc/diver.f03:25-27): rhs = div(uc, vc, wc) / dt;
* gradie (fsrc/gradie.f03:30-116): the Cartesian pressure gradient at the
  cell centres times -dt/2 J^-1 from the face normals csx..ztz, and the
  contravariant gradient on the faces from the metric g11..g33;
* vel_up (fsrc/vel_up.f03:40-52, 188-285): u += gra, uc -= dt cgra1 on
  i = 0..jx, vc -= dt cgra2 on j = 1..jy-1, wc -= dt cgra3 on k = 0..jz.

The face normals J grad(csi) etc. are restated from metrica.f03 (:158-160,
:272-276, and the zeta faces) on the ghosted node coordinates of the C
oracle (cellep's ghost nodes); they are pinned by rebuilding g11, g22, g33
from them and the face Jacobians and comparing with the C oracle's metric.
"""

from __future__ import annotations

import numpy as np


def _node_views(orc):
    X, Y, Z = (orc.coords(c) for c in range(3))  # (-8:jx+8, -8:jy+8, -8:jz+8)
    o = 8
    return (lambda a, b, c: X[a + o, b + o, c + o], lambda a, b, c: Y[a + o, b + o, c + o],
            lambda a, b, c: Z[a + o, b + o, c + o])


def _jac(xc, yc, zc, xe, ye, ze, xz, yz, zz):
    return xc * (ye * zz - yz * ze) - xe * (yc * zz - yz * zc) + xz * (yc * ze - ye * zc)


def face_normals(orc):
    """Returns (csi, eta, zeta) triples of face-normal arrays with the extents
    of g1*, g2*, g3* and the face Jacobians: ((csx, csy, csz, J), ...)."""
    jx, jy, jz = orc.jx, orc.jy, orc.jz
    Xf, Yf, Zf = _node_views(orc)
    # csi faces i = 0..jx, j = 1..jy, k = 1..jz
    i = np.arange(0, jx + 1)[:, None, None]
    j = np.arange(1, jy + 1)[None, :, None]
    k = np.arange(1, jz + 1)[None, None, :]
    j2, j1, k2, k1 = j, j - 1, k, k - 1

    def avg_i(F, a):
        return .25 * (F(a, j2, k2) + F(a, j2, k1) + F(a, j1, k2) + F(a, j1, k1))

    d = {}
    for nm, F in (("x", Xf), ("y", Yf), ("z", Zf)):
        d[nm + "csi"] = .5 * (avg_i(F, i + 1) - avg_i(F, i - 1))
        d[nm + "eta"] = .5 * (F(i, j2, k2) + F(i, j2, k1)) - .5 * (F(i, j1, k2) + F(i, j1, k1))
        d[nm + "zet"] = .5 * (F(i, j2, k2) + F(i, j1, k2)) - .5 * (F(i, j2, k1) + F(i, j1, k1))
    csx = d["yeta"] * d["zzet"] - d["yzet"] * d["zeta"]
    csy = d["xzet"] * d["zeta"] - d["xeta"] * d["zzet"]
    csz = d["xeta"] * d["yzet"] - d["xzet"] * d["yeta"]
    Jc = _jac(*(d[a + b] for b in ("csi", "eta", "zet") for a in "xyz"))
    # eta faces i = 1..jx, j = 0..jy, k = 1..jz (one-sided at the walls)
    i = np.arange(1, jx + 1)[:, None, None]
    jj = np.arange(0, jy + 1)
    k = np.arange(1, jz + 1)[None, None, :]
    i2, i1, k2, k1 = i, i - 1, k, k - 1

    def avg_j(F, b):
        b = np.asarray(b)[None, :, None]
        return .25 * (F(i2, b, k2) + F(i2, b, k1) + F(i1, b, k1) + F(i1, b, k2))

    e = {}
    jc = jj[None, :, None]
    for nm, F in (("x", Xf), ("y", Yf), ("z", Zf)):
        interior = .5 * (avg_j(F, np.clip(jj + 1, 0, jy)) - avg_j(F, np.clip(jj - 1, 0, jy)))
        lo = .5 * (-3. * avg_j(F, np.zeros_like(jj)) + 4. * avg_j(F, np.ones_like(jj)) - avg_j(F, np.full_like(jj, 2)))
        hi = .5 * (3. * avg_j(F, np.full_like(jj, jy)) - 4. * avg_j(F, np.full_like(jj, jy - 1))
                   + avg_j(F, np.full_like(jj, jy - 2)))
        eta = np.where(jc == 0, lo, np.where(jc == jy, hi, interior))
        e[nm + "eta"] = eta
        e[nm + "csi"] = .5 * (F(i2, jc, k2) + F(i2, jc, k1)) - .5 * (F(i1, jc, k2) + F(i1, jc, k1))
        e[nm + "zet"] = .5 * (F(i2, jc, k2) + F(i1, jc, k2)) - .5 * (F(i2, jc, k1) + F(i1, jc, k1))
    etx = e["yzet"] * e["zcsi"] - e["ycsi"] * e["zzet"]
    ety = e["xcsi"] * e["zzet"] - e["xzet"] * e["zcsi"]
    etz = e["xzet"] * e["ycsi"] - e["xcsi"] * e["yzet"]
    Je = _jac(*(e[a + b] for b in ("csi", "eta", "zet") for a in "xyz"))
    # zeta faces i = 1..jx, j = 1..jy, k = 0..jz
    i = np.arange(1, jx + 1)[:, None, None]
    j = np.arange(1, jy + 1)[None, :, None]
    k = np.arange(0, jz + 1)[None, None, :]
    i2, i1, j2, j1 = i, i - 1, j, j - 1

    def avg_k(F, c):
        return .25 * (F(i2, j2, c) + F(i2, j1, c) + F(i1, j1, c) + F(i1, j2, c))

    z = {}
    for nm, F in (("x", Xf), ("y", Yf), ("z", Zf)):
        z[nm + "zet"] = .5 * (avg_k(F, k + 1) - avg_k(F, k - 1))
        z[nm + "csi"] = .5 * (F(i2, j2, k) + F(i2, j1, k)) - .5 * (F(i1, j2, k) + F(i1, j1, k))
        z[nm + "eta"] = .5 * (F(i2, j2, k) + F(i1, j2, k)) - .5 * (F(i2, j1, k) + F(i1, j1, k))
    ztx = z["ycsi"] * z["zeta"] - z["yeta"] * z["zcsi"]
    zty = z["xeta"] * z["zcsi"] - z["xcsi"] * z["zeta"]
    ztz = z["xcsi"] * z["yeta"] - z["xeta"] * z["ycsi"]
    Jz = _jac(*(z[a + b] for b in ("csi", "eta", "zet") for a in "xyz"))
    return (csx, csy, csz, Jc), (etx, ety, etz, Je), (ztx, zty, ztz, Jz)


def contra(orc, u, v, w, vc_old):
    """Returns (uc, vc, wc, cs3, cs4) from the cell-centred u, v, w
    (jx+2, jy+2, jz+2) and the previous vc, whose wall faces give the old
    wall fluxes; cs3, cs4 are (jx, jz).  Periodic x and z."""
    uc, vc, wc, cs = contra_walls(orc, u, v, w, None, vc_old, None)
    return uc, vc, wc, cs[2], cs[3]


def contra_walls(orc, u, v, w, uc_old, vc_old, wc_old):
    """contra with the grid's periodicity (orc.ip, orc.kp): the faces of a
    walled direction take the wall velocity of the ghost cell and give
    cs = new minus old wall flux (contra.f03:34-67 x walls, 160-190 z walls,
    several-rank form).  Returns (uc, vc, wc, [cs1..cs6]) with zero arrays
    for periodic directions."""
    jx, jy, jz = orc.jx, orc.jy, orc.jz
    (csx, csy, csz, _), (etx, ety, etz, _), (ztx, zty, ztz, _) = face_normals(orc)

    def avg(a, s0, s1):
        return .5 * (a[s0] + a[s1])

    si0, si1 = np.s_[0:jx + 1, 1:jy + 1, 1:jz + 1], np.s_[1:jx + 2, 1:jy + 1, 1:jz + 1]
    uc = avg(u, si0, si1) * csx + avg(v, si0, si1) * csy + avg(w, si0, si1) * csz
    vc = np.empty((jx, jy + 1, jz))
    sj0, sj1 = np.s_[1:jx + 1, 1:jy, 1:jz + 1], np.s_[1:jx + 1, 2:jy + 1, 1:jz + 1]
    vc[:, 1:jy] = (avg(u, sj0, sj1) * etx[:, 1:jy] + avg(v, sj0, sj1) * ety[:, 1:jy]
                   + avg(w, sj0, sj1) * etz[:, 1:jy])
    cs = [np.zeros((jy, jz)), np.zeros((jy, jz)), None, None, np.zeros((jx, jy)), np.zeros((jx, jy))]
    for s, (jf, jw) in enumerate(((0, 0), (jy, jy + 1))):
        flux = (u[1:jx + 1, jw, 1:jz + 1] * etx[:, jf] + v[1:jx + 1, jw, 1:jz + 1] * ety[:, jf]
                + w[1:jx + 1, jw, 1:jz + 1] * etz[:, jf])
        cs[2 + s] = flux - vc_old[:, jf]
        vc[:, jf] = flux
    if orc.ip == 1:
        for s, (iff, iw) in enumerate(((0, 0), (jx, jx + 1))):
            flux = (u[iw, 1:jy + 1, 1:jz + 1] * csx[iff] + v[iw, 1:jy + 1, 1:jz + 1] * csy[iff]
                    + w[iw, 1:jy + 1, 1:jz + 1] * csz[iff])
            cs[s] = flux - uc_old[iff]
            uc[iff] = flux
    sk0, sk1 = np.s_[1:jx + 1, 1:jy + 1, 0:jz + 1], np.s_[1:jx + 1, 1:jy + 1, 1:jz + 2]
    wc = avg(u, sk0, sk1) * ztx + avg(v, sk0, sk1) * zty + avg(w, sk0, sk1) * ztz
    if orc.kp == 1:
        for s, (kf, kw) in enumerate(((0, 0), (jz, jz + 1))):
            flux = (u[1:jx + 1, 1:jy + 1, kw] * ztx[:, :, kf] + v[1:jx + 1, 1:jy + 1, kw] * zty[:, :, kf]
                    + w[1:jx + 1, 1:jy + 1, kw] * ztz[:, :, kf])
            cs[4 + s] = flux - wc_old[:, :, kf]
            wc[:, :, kf] = flux
    return uc, vc, wc, cs


def diver(uc, vc, wc, dt):
    """rhs (jx, jy, jz) from uc (jx+1, jy, jz), vc (jx, jy+1, jz), wc (jx, jy, jz+1)."""
    return (uc[1:] - uc[:-1] + vc[:, 1:] - vc[:, :-1] + wc[:, :, 1:] - wc[:, :, :-1]) / dt


def project(orc, fi, uc, vc, wc, u, v, w, dt):
    """vel_up after gradie for the pressure fi (jx+2, jy+2, jz+2) with its
    ghost layer; returns new (uc, vc, wc, u, v, w)."""
    jx, jy, jz = orc.jx, orc.jy, orc.jz
    g = {n: orc.metric(1, n) for n in ("g11", "g12", "g13", "g21", "g22", "g23", "g31", "g32", "g33", "giac")}
    P = fi

    def p(di, dj, dk, i0, i1, j0, j1, k0, k1):  # fi over an index box shifted by (di,dj,dk)
        return P[i0 + di:i1 + di + 1, j0 + dj:j1 + dj + 1, k0 + dk:k1 + dk + 1]

    # cgra1 on i = 0..jx, j = 1..jy, k = 1..jz
    b = (0, jx, 1, jy, 1, jz)
    cg1 = (g["g11"] * (p(1, 0, 0, *b) - p(0, 0, 0, *b))
           + .25 * g["g12"] * (p(1, 1, 0, *b) + p(0, 1, 0, *b) - p(1, -1, 0, *b) - p(0, -1, 0, *b))
           + .25 * g["g13"] * (p(1, 0, 1, *b) + p(0, 0, 1, *b) - p(1, 0, -1, *b) - p(0, 0, -1, *b)))
    b = (1, jx, 0, jy, 1, jz)
    cg2 = (g["g22"] * (p(0, 1, 0, *b) - p(0, 0, 0, *b))
           + .25 * g["g21"] * (p(1, 1, 0, *b) + p(1, 0, 0, *b) - p(-1, 1, 0, *b) - p(-1, 0, 0, *b))
           + .25 * g["g23"] * (p(0, 1, 1, *b) + p(0, 0, 1, *b) - p(0, 1, -1, *b) - p(0, 0, -1, *b)))
    b = (1, jx, 1, jy, 0, jz)
    cg3 = (g["g33"] * (p(0, 0, 1, *b) - p(0, 0, 0, *b))
           + .25 * g["g31"] * (p(1, 0, 1, *b) + p(1, 0, 0, *b) - p(-1, 0, 1, *b) - p(-1, 0, 0, *b))
           + .25 * g["g32"] * (p(0, 1, 1, *b) + p(0, 1, 0, *b) - p(0, -1, 1, *b) - p(0, -1, 0, *b)))
    # wall faces keep their flux (vel_up.f03:188-285)
    i0, i1 = (0, jx + 1) if orc.ip == 0 else (1, jx)
    k0, k1 = (0, jz + 1) if orc.kp == 0 else (1, jz)
    uc2 = uc.copy()
    uc2[i0:i1] -= dt * cg1[i0:i1]
    vc2 = vc.copy()
    vc2[:, 1:jy] -= dt * cg2[:, 1:jy]
    wc2 = wc.copy()
    wc2[:, :, k0:k1] -= dt * cg3[:, :, k0:k1]
    out = [uc2, vc2, wc2]
    if u is not None:
        (csx, csy, csz, _), (etx, ety, etz, _), (ztx, zty, ztz, _) = face_normals(orc)
        c = P[1:-1, 1:-1, 1:-1]
        se, sw = c + P[2:, 1:-1, 1:-1], c + P[:-2, 1:-1, 1:-1]
        sn, ss = c + P[1:-1, 2:, 1:-1], c + P[1:-1, :-2, 1:-1]
        sf, sb = c + P[1:-1, 1:-1, 2:], c + P[1:-1, 1:-1, :-2]
        coef = -0.5 * dt / g["giac"]
        res = []
        for cs, et, zt, a in ((csx, etx, ztx, u), (csy, ety, zty, v), (csz, etz, ztz, w)):
            gr = coef * (cs[1:] * se - cs[:-1] * sw + et[:, 1:] * sn - et[:, :-1] * ss + zt[:, :, 1:] * sf
                         - zt[:, :, :-1] * sb)
            a2 = a.copy()
            a2[1:-1, 1:-1, 1:-1] += gr
            if orc.ip == 0:  # periodic images (vel_up.f03:82-100)
                a2[0, 1:-1, 1:-1] = a2[jx, 1:-1, 1:-1]
                a2[jx + 1, 1:-1, 1:-1] = a2[1, 1:-1, 1:-1]
            if orc.kp == 0:
                a2[:, 1:-1, 0] = a2[:, 1:-1, jz]
                a2[:, 1:-1, jz + 1] = a2[:, 1:-1, 1]
            res.append(a2)
        out += res
    return out
