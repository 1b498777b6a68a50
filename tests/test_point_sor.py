"""The multicolour point SOR (smoother 3, the reference's islor = 0:
solut_sndrcv_sor, multigrid.f03:656-1010) and the free surface of the top
wall (mul_boun_sndrcv, multigrid.f03:1188-1222), through the C ABI, against
the oracle's restatement of the reference's point SOR.

Tolerances: solves converged to ||r||/||b|| <= 1e-12 agree with the oracle's
converged solution within 1e-8 in the L2 and max norms (zero-mean fields
without a free surface; the fields themselves with one, where the pressure
level is fixed).  On the uniform sample deck the free-surface relation has
no cross terms, so the two cells either side of the surface average to the
given surface pressure: checked to 1e-9 of its size.
"""
import json
import os

import numpy as np
import pytest

from oracle.oracle import Oracle
from ples_gb300 import mg
from ples_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

SOL_TOL = 1e-8


def _deck():
    d = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "sample_deck.json")))
    xs, ys, zs = (np.array(d[c]) for c in "xyz")
    shp = (xs.size, ys.size, zs.size)
    x = np.asfortranarray(np.broadcast_to(xs[:, None, None], shp))
    y = np.asfortranarray(np.broadcast_to(ys[None, :, None], shp))
    z = np.asfortranarray(np.broadcast_to(zs[None, None, :], shp))
    return d, xs, zs, x, y, z


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b), np.abs(a - b).max() / np.abs(b).max()


def _zm(fi):
    p = fi[1:-1, 1:-1, 1:-1]
    return p - p.mean()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_point_sor_on_the_sample_deck(precision):
    d, xs, zs, x, y, z = _deck()
    jx, jy, jz = d["dims"]
    rhs = S.divergence_rhs(jx, jy, jz, seed=0)
    orc = Oracle(x, y, z, islor=0, omega=1.6, nlevmax=4, nproc=2)
    fo, cyc, _, rr = orc.multi(rhs, eps=1e-13, ficycle=2000)
    assert rr <= 1e-13
    with mg.Multigrid(x, y, z, precision=precision, smoother=3, omega=1.6, nlevmax=4) as m:
        fi, st = m.solve(rhs, rel_tol=1e-12, max_cycles=200)
    assert st["status"] == mg.OK, st
    l2, mx = _rel(_zm(fi), _zm(fo))
    assert l2 <= SOL_TOL and mx <= SOL_TOL, (l2, mx)


def test_point_sor_on_a_curvilinear_grid():
    dims = (32, 16, 32)
    x, y, z = S.wavy_channel_grid(*dims, 0.03, 1.3)
    rhs = S.divergence_rhs(*dims, seed=21)
    fo, *_ = Oracle(x, y, z, islor=1).multi(rhs, eps=1e-13, ficycle=400)
    with mg.Multigrid(x, y, z, smoother=3) as m:
        fi, st = m.solve(rhs, rel_tol=1e-12, max_cycles=300)
        assert st["status"] == mg.OK, st
    l2, mx = _rel(_zm(fi), _zm(fo))
    assert l2 <= SOL_TOL and mx <= SOL_TOL, (l2, mx)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_free_surface_on_the_sample_deck(precision):
    d, xs, zs, x, y, z = _deck()
    jx, jy, jz = d["dims"]
    rhs = S.divergence_rhs(jx, jy, jz, seed=0)
    xc, zc = 0.5 * (xs[:-1] + xs[1:]), 0.5 * (zs[:-1] + zs[1:])
    prs = np.asfortranarray(0.3 * np.sin(xc)[:, None] * np.cos(3 * zc)[None, :] + 0.1)
    orc = Oracle(x, y, z, islor=0, omega=1.6, nlevmax=4, nproc=2)
    orc.set_free_surface(True, prs)
    fo, _, _, rr = orc.multi(rhs, eps=1e-13, ficycle=2000)
    assert rr <= 1e-13
    with mg.Multigrid(x, y, z, precision=precision, smoother=3, omega=1.6, nlevmax=4, freesurface=1) as m:
        m.set_surface_pressure(prs)
        fi, st = m.solve(rhs, rel_tol=1e-12, max_cycles=200)
    assert st["status"] == mg.OK, st
    assert st["rhs_mean_removed"] == 0.0  # the pressure level is fixed: no compatibility shift
    # the fields themselves agree: no null space to remove
    l2, mx = _rel(fi[1:-1, 1:-1, 1:-1], fo[1:-1, 1:-1, 1:-1])
    assert l2 <= SOL_TOL and mx <= SOL_TOL, (l2, mx)
    surf = 0.5 * (fi[1:-1, jy, 1:-1] + fi[1:-1, jy + 1, 1:-1])
    assert np.abs(surf - prs).max() <= 1e-9 * np.abs(prs).max()


def test_free_surface_first_step_on_a_curvilinear_grid():
    """next_prs not given (the reference's first time step, PrS0 = 0), on a
    grid whose metric has cross terms at the surface."""
    dims = (32, 16, 32)
    x, y, z = S.wavy_channel_grid(*dims, 0.03, 1.3)
    rhs = S.divergence_rhs(*dims, seed=22)
    orc = Oracle(x, y, z, islor=0, omega=1.2, nlevmax=4)
    orc.set_free_surface(True, None)
    fo, _, _, rr = orc.multi(rhs, eps=1e-13, ficycle=3000)
    assert rr <= 1e-13
    with mg.Multigrid(x, y, z, smoother=3, freesurface=1) as m:
        fi, st = m.solve(rhs, rel_tol=1e-12, max_cycles=300)
    assert st["status"] == mg.OK, st
    l2, mx = _rel(fi[1:-1, 1:-1, 1:-1], fo[1:-1, 1:-1, 1:-1])
    assert l2 <= SOL_TOL and mx <= SOL_TOL, (l2, mx)


def test_free_surface_setter_needs_a_free_surface_handle():
    d, xs, zs, x, y, z = _deck()
    with mg.Multigrid(x, y, z, smoother=3, nlevmax=4) as m:
        with pytest.raises(mg.PlesMGError):
            m.set_surface_pressure(np.zeros((d["dims"][0], d["dims"][2])))
