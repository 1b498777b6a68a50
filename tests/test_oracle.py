"""Pins the CPU oracle (the restated PLES multigrid) with known answers.

The reference has no tests of its own; its only fixture is the sample deck
(tests/golden/sample_deck.json, made from gri3dp_in.dat).  These checks pin
the restatement: exact metric values on that deck at every level, an exact
spectral solution of the discrete problem on a uniform grid, second-order
consistency on a curvilinear grid, flux conservation with the wall ghost
relation, transfer-operator identities, and independence of the converged
solution from the emulated rank count and the smoother.
"""
import hashlib
import json
import math
import os

import numpy as np
import pytest
import scipy.fft as sfft

from oracle.oracle import Oracle
from ples_gb300 import synthetic as S

GOLD = os.path.join(os.path.dirname(__file__), "golden", "sample_deck.json")


def sample_deck():
    d = json.load(open(GOLD))
    xs, ys, zs = (np.array(d[c]) for c in "xyz")
    shape = (xs.size, ys.size, zs.size)
    x = np.asfortranarray(np.broadcast_to(xs[:, None, None], shape))
    y = np.asfortranarray(np.broadcast_to(ys[None, :, None], shape))
    z = np.asfortranarray(np.broadcast_to(zs[None, None, :], shape))
    return d, x, y, z


def test_sample_deck_reconstruction_matches_checksum():
    d, x, y, z = sample_deck()
    h = hashlib.sha256()
    for a in (x, y, z):
        h.update(np.ascontiguousarray(a.ravel(order="F")).tobytes())
    assert h.hexdigest() == d["coords_sha256"]
    assert list(x.shape) == [n + 1 for n in d["dims"]]


def _periodic_nodes(v, s, lo, hi):
    """Node planes v(m*s) for m in [lo, hi] with the cellep periodic shift."""
    n = v.size - 1
    out = []
    for m in range(lo, hi + 1):
        q = m * s
        if q < 0:
            out.append(v[0] - (v[n] - v[n + q]))
        elif q > n:
            out.append(v[n] - (v[0] - v[q - n]))
        else:
            out.append(v[q])
    return np.array(out)


@pytest.mark.parametrize("level", [1, 2, 3, 4])
def test_sample_deck_metric_known_answer(level):
    """Tensor-product grid: g11 = Y'Z'/X', g22 = X'Z'/Y', g33 = X'Y'/Z',
    cross terms zero up to the rounding of the one-sided wall formula
    0.5*(-3a + 4a - a) (metrica.f03, mul_met in multigrid.f03)."""
    d, x, y, z = sample_deck()
    o = Oracle(x, y, z, ip=0, jp=1, kp=0)
    assert o.nlevel == 4
    s = 2 ** (level - 1)
    nx, ny, nz = o.dims(level)
    xs, ys, zs = x[:, 0, 0], y[0, :, 0], z[0, 0, :]
    X = _periodic_nodes(xs, s, -1, nx + 1)  # index m -> X[m + 1]
    Z = _periodic_nodes(zs, s, -1, nz + 1)
    Y = ys[::s]
    dX = X[2:-1] - X[1:-2]          # cell widths, i = 1..nx
    dZ = Z[2:-1] - Z[1:-2]
    dY = Y[1:] - Y[:-1]
    Xc = 0.5 * (X[2:] - X[:-2])     # face-centred, i = 0..nx
    Zc = 0.5 * (Z[2:] - Z[:-2])
    Yc = np.empty(ny + 1)
    Yc[1:-1] = 0.5 * (Y[2:] - Y[:-2])
    Yc[0] = 0.5 * (-3 * Y[0] + 4 * Y[1] - Y[2])
    Yc[-1] = 0.5 * (3 * Y[-1] - 4 * Y[-2] + Y[-3])
    g11 = (dY[None, :, None] * dZ[None, None, :]) / Xc[:, None, None] / s
    g22 = (dX[:, None, None] * dZ[None, None, :]) / Yc[None, :, None] / s
    g33 = (dX[:, None, None] * dY[None, :, None]) / Zc[None, None, :] / s
    np.testing.assert_allclose(o.metric(level, "g11"), g11, rtol=1e-12)
    np.testing.assert_allclose(o.metric(level, "g22"), g22, rtol=1e-12)
    np.testing.assert_allclose(o.metric(level, "g33"), g33, rtol=1e-12)
    scale = max(np.abs(g11).max(), np.abs(g22).max(), np.abs(g33).max())
    for c in ("g12", "g13", "g21", "g23", "g31", "g32"):
        assert np.abs(o.metric(level, c)).max() <= 1e-14 * scale
    if level == 1:
        giac = dX[:, None, None] * dY[None, :, None] * dZ[None, None, :]
        np.testing.assert_allclose(o.metric(1, "giac"), giac, rtol=1e-12)


def spectral_solution(rhs, g11, g22, g33):
    """Exact solution of the uniform-grid discrete problem: periodic x and z
    (DFT), zero-flux y walls with mirror ghosts (DCT-II); zero mean."""
    jx, jy, jz = rhs.shape
    lx = 2 * (np.cos(2 * np.pi * np.arange(jx) / jx) - 1)
    ly = 2 * (np.cos(np.pi * np.arange(jy) / jy) - 1)
    lz = 2 * (np.cos(2 * np.pi * np.arange(jz) / jz) - 1)
    lam = g11 * lx[:, None, None] + g22 * ly[None, :, None] + g33 * lz[None, None, :]
    bh = sfft.dct(np.fft.fftn(rhs, axes=(0, 2)), type=2, axis=1, norm="ortho")
    lam[0, 0, 0] = 1.0
    ph = bh / lam
    ph[0, 0, 0] = 0.0
    p = np.real(np.fft.ifftn(sfft.idct(ph, type=2, axis=1, norm="ortho"), axes=(0, 2)))
    return p - p.mean()


@pytest.mark.parametrize("islor", [0, 1])
def test_uniform_grid_solution_matches_spectral(islor):
    jx, jy, jz = 32, 16, 32
    lx, ly, lz = 2 * math.pi, 2.0, 2 * math.pi / 3
    x, y, z = S.uniform_grid(jx, jy, jz, lx, ly, lz)
    o = Oracle(x, y, z, islor=islor)
    rhs = S.divergence_rhs(jx, jy, jz, seed=7)
    fi, cyc, rm, rr = o.multi(rhs, eps=1e-13, ficycle=200)
    assert rr <= 1e-13
    p = fi[1:-1, 1:-1, 1:-1]
    p = p - p.mean()
    dx, dy, dz = lx / jx, ly / jy, lz / jz
    ref = spectral_solution(rhs, dy * dz / dx, dx * dz / dy, dx * dy / dz)
    err = np.linalg.norm(p - ref) / np.linalg.norm(ref)
    assert err < 1e-10, err


def _centroids(o):
    X, Y, Z = (o.coords(c) for c in range(3))  # (-8:jx+8, ...)
    def cc(a):
        return 0.125 * (a[:-1, :-1, :-1] + a[1:, :-1, :-1] + a[:-1, 1:, :-1] + a[:-1, :-1, 1:]
                        + a[1:, 1:, :-1] + a[1:, :-1, 1:] + a[:-1, 1:, 1:] + a[1:, 1:, 1:])
    # cell (i,j,k) spans nodes i-1..i -> index i+7 in the centroid arrays
    return cc(X), cc(Y), cc(Z)


def _consistency_error(jx, jy, jz):
    x, y, z = S.wavy_channel_grid(jx, jy, jz, 0.05, 1.0)
    o = Oracle(x, y, z)
    cx, cy, cz = _centroids(o)
    sl = (slice(7, 7 + jx + 2), slice(7, 7 + jy + 2), slice(7, 7 + jz + 2))
    X, Y, Z = cx[sl], cy[sl], cz[sl]
    p = np.cos(X) * np.cos(2 * Z) * Y ** 2
    lap = np.cos(X) * np.cos(2 * Z) * (2 - 5 * Y ** 2)
    L = o.resid(1, np.asfortranarray(p), np.zeros((jx, jy, jz), order="F"))
    giac = o.metric(1, "giac")
    err = (L / giac - lap[1:-1, 1:-1, 1:-1])[:, 1:-1, :]  # skip wall-adjacent rows
    return np.abs(err).max()


def test_curvilinear_operator_second_order():
    e1 = _consistency_error(32, 16, 32)
    e2 = _consistency_error(64, 32, 64)
    assert e2 < e1 / 3.0, (e1, e2)


def test_wall_ghost_relation_conserves_flux():
    """With the ghosts at the fixed point of mul_boun_sndrcv and zero wall
    fluxes, the residual operator sums to zero over the domain."""
    w = S.WORKLOADS["channel_64x32x64"]
    x, y, z = S.wavy_channel_grid(32, 16, 32, w.amp, w.beta)
    o = Oracle(x, y, z)
    rng = np.random.default_rng(3)
    pr = np.asfortranarray(rng.standard_normal((34, 18, 34)))
    for _ in range(6):
        pr = o.ghost_fill(1, pr)
    L = o.resid(1, pr, np.zeros((32, 16, 32), order="F"))
    assert abs(L.sum()) < 1e-12 * np.abs(L).sum()
    # constants are in the null space
    c = np.full((34, 18, 34), 3.25, order="F")
    c = o.ghost_fill(1, c)
    assert np.all(c == 3.25)
    assert np.all(o.resid(1, c, np.zeros((32, 16, 32), order="F")) == 0.0)


def test_transfer_identities():
    x, y, z = S.wavy_channel_grid(32, 16, 32, 0.05, 2.0)
    o = Oracle(x, y, z)
    rng = np.random.default_rng(5)
    r = np.asfortranarray(rng.standard_normal((32, 16, 32)))
    rc = o.restrict(1, r)
    np.testing.assert_allclose(rc.sum(), -r.sum() / 8.0, atol=1e-12)
    np.testing.assert_allclose(rc[0, 0, 0], -r[0:2, 0:2, 0:2].sum() / 8.0, rtol=1e-14)
    fine = np.zeros((34, 18, 34), order="F")
    coarse = np.full((18, 10, 18), 2.0, order="F")
    out = o.prolong(1, fine, coarse)
    assert np.all(out == 2.0)


def test_rank_emulation_converges_to_same_solution():
    w = S.WORKLOADS["channel_64x32x64"]
    x, y, z = S.wavy_channel_grid(32, 16, 32, w.amp, w.beta)
    rhs = S.divergence_rhs(32, 16, 32, seed=11)
    sols = []
    for nproc in (1, 2, 4):
        o = Oracle(x, y, z, islor=1, nproc=nproc)
        fi, cyc, rm, rr = o.multi(rhs, eps=1e-13, ficycle=200)
        assert rr <= 1e-13
        p = fi[1:-1, 1:-1, 1:-1]
        sols.append(p - p.mean())
    for s in sols[1:]:
        assert np.linalg.norm(s - sols[0]) / np.linalg.norm(sols[0]) < 1e-10


def test_point_sor_diverges_on_stretched_channel_but_line_sor_converges():
    """The reference's default smoother (point SOR, omega = 1.6) diverges on
    the stretched wavy channel; its line-SOR option converges."""
    w = S.WORKLOADS["channel_64x32x64"]
    x, y, z = w.grid()
    rhs = w.rhs()
    _, _, _, rr10 = Oracle(x, y, z, islor=0).multi(rhs, eps=1e-10, ficycle=10)
    _, _, _, rr40 = Oracle(x, y, z, islor=0).multi(rhs, eps=1e-10, ficycle=40)
    _, cyc, _, rr_slor = Oracle(x, y, z, islor=1).multi(rhs, eps=1e-10, ficycle=60)
    assert rr40 > 5.0 * rr10 > 1e-3
    assert rr_slor <= 1e-10 and cyc < 30


def test_line_sor_diverges_with_x_walls_on_wavy_stretched_channel():
    """With walls in x (ip = 1) on a wavy (A = 0.1), strongly stretched
    (beta = 2.5) channel the reference's own line-SOR multigrid ends in NaN,
    as it does with walls in x and z; the same grid with z walls only, or
    with milder stretching, converges.  The device solver reports this case
    as diverged (tests/test_walls.py)."""
    dims = (64, 32, 64)
    x, y, z = S.wavy_channel_grid(*dims, 0.1, 2.5)
    rhs = S.divergence_rhs(*dims, seed=4)
    for ip, kp, npr in ((1, 0, 1), (1, 1, 2)):
        _, _, _, rr = Oracle(x, y, z, ip=ip, kp=kp, islor=1, nproc=npr).multi(rhs, eps=1e-10, ficycle=200)
        assert not np.isfinite(rr), (ip, kp, rr)
    _, _, _, rr = Oracle(x, y, z, ip=0, kp=1, islor=1, nproc=2).multi(rhs, eps=1e-10, ficycle=200)
    assert rr <= 1e-10
    x, y, z = S.wavy_channel_grid(*dims, 0.1, 1.0)
    _, _, _, rr = Oracle(x, y, z, ip=1, kp=0, islor=1).multi(rhs, eps=1e-10, ficycle=200)
    assert rr <= 1e-10


def test_bad_arguments_rejected():
    x, y, z = S.wavy_channel_grid(32, 16, 32, 0.05, 2.0)
    with pytest.raises(ValueError):
        Oracle(x, y, z, jp=0)
    with pytest.raises(ValueError):
        Oracle(x, y, z, nproc=3)
