"""Immersed-boundary mask: solid cells removed from the pressure system
(no counterpart in the reference's multigrid; oracle/masked.py restates the
reference's fine-level system and extends it with the mask).

Tolerances: the masked assembly with an empty mask reproduces the restated
reference solver's converged solution to 1e-9 (the pin); device solves
converge to ||r||/||b|| <= 1e-10 and agree with the masked oracle's exact
solution to 1e-8 (zero-mean over fluid cells, L2 and max, relative); the
solution is exactly zero on solid cells.
"""
import numpy as np
import pytest

from oracle.masked import solve as masked_solve
from oracle.oracle import Oracle
from ples_gb300 import synthetic as S

DIMS = (32, 16, 32)


@pytest.fixture(scope="module")
def case():
    x, y, z = S.wavy_channel_grid(*DIMS, 0.08, 2.0)
    rhs = S.divergence_rhs(*DIMS, seed=12)
    solid = S.sphere_mask(x, y, z, n=6, rmin=0.3, rmax=0.5, seed=3)
    return dict(x=x, y=y, z=z, rhs=rhs, solid=solid, orc=Oracle(x, y, z, islor=1))


def _zm(p, fluid):
    return np.where(fluid, p - p[fluid].mean(), 0.0)


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b), np.abs(a - b).max() / np.abs(b).max()


def test_mask_has_solid_and_fluid(case):
    s = case["solid"]
    assert 0.01 < s.mean() < 0.5


def test_empty_mask_assembly_matches_reference_solver(case):
    fi, cyc, rm, rr = case["orc"].multi(case["rhs"], eps=1e-13, ficycle=400)
    assert rr <= 1e-12
    ref = fi[1:-1, 1:-1, 1:-1]
    p = masked_solve(case["orc"], case["rhs"])
    fluid = np.ones(DIMS, dtype=bool)
    l2, mx = _rel(_zm(p, fluid), _zm(ref, fluid))
    assert l2 <= 1e-9 and mx <= 1e-9, (l2, mx)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["mixed", "fp64", "mixed-64-line-tiles"])
def test_device_masked_solve_matches_oracle(case, precision):
    from ples_gb300 import mg
    ref = masked_solve(case["orc"], case["rhs"], case["solid"])
    fluid = ~case["solid"]
    prec = precision.split("-")[0]
    with mg.Multigrid(case["x"], case["y"], case["z"], precision=prec, solid=case["solid"]) as m:
        if precision.endswith("tiles"):  # the 64-line-tile smoother at every level with nx even
            for lev in range(1, m.nlevel + 1):
                nx, _, nz = m.dims(lev)
                if nx % 2 == 0 and nz >= 2:
                    m.set_line_threads(lev, 1024)
        fi, st = m.solve(case["rhs"], rel_tol=1e-10, max_cycles=300)
    assert st["status"] == mg.OK and st["rel_residual"] <= 1e-10, st
    p = fi[1:-1, 1:-1, 1:-1]
    assert np.all(p[case["solid"]] == 0.0)
    l2, mx = _rel(_zm(p, fluid), _zm(ref, fluid))
    assert l2 <= 1e-8 and mx <= 1e-8, (l2, mx)


def test_vectorised_masked_residual_matches_assembly():
    """oracle.masked.residual (used at the 512x256x512 size, where the sparse
    assembly does not fit) against the assembled matrix times the field, and
    without a mask against the C oracle's residual: interior rows to 1e-14;
    the wall rows are the flux through the wall face (the assembly's bottom
    row carries it with the opposite sign)."""
    from oracle import masked as M
    nx, ny, nz = 24, 12, 16
    x, y, z = S.wavy_channel_grid(nx, ny, nz, 0.08, 2.0)
    rhs = S.divergence_rhs(nx, ny, nz, seed=12)
    orc = Oracle(x, y, z, islor=1)
    fi = np.asfortranarray(np.random.default_rng(0).standard_normal((nx + 2, ny + 2, nz + 2)))
    p = fi.copy(order="F")
    p[0], p[nx + 1] = p[nx], p[1]
    p[:, :, 0], p[:, :, nz + 1] = p[:, :, nz], p[:, :, 1]
    r, _ = M.residual(orc, fi, rhs)
    rc = orc.resid(1, p, rhs - rhs.mean())
    assert np.abs(r - rc).max() <= 1e-14 * np.abs(rc).max()
    solid = S.sphere_mask(x, y, z, n=4, rmin=0.3, rmax=0.5, seed=3)
    r, rw = M.residual(orc, fi, rhs, solid)
    c = M.apply_mask(M._coef_boxes(orc, nx, ny, nz), M.mask_box(solid, nx, ny, nz))
    ident = np.zeros((nx, ny + 2, nz), dtype=bool)
    ident[:, 1:ny + 1, :] = solid
    ident[:, 0, :], ident[:, ny + 1, :] = solid[:, 0, :], solid[:, -1, :]
    A, _, unk = M.assemble(c, nx, ny, nz, ident)
    I, J, K = np.meshgrid(np.arange(1, nx + 1), np.arange(0, ny + 2), np.arange(1, nz + 1), indexing="ij")
    xv = np.zeros(A.shape[0])
    xv[unk(I, J, K).ravel()] = p[1:nx + 1, :, 1:nz + 1].ravel()
    Ax = A @ xv
    fl = ~solid
    b = np.where(fl, rhs, 0.0)
    b = np.where(fl, b - b[fl].mean(), 0.0)
    I, J, K = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1), np.arange(1, nz + 1), indexing="ij")
    ra = np.where(solid, 0.0, Ax[unk(I, J, K)] - b)
    assert np.abs(r - ra).max() <= 1e-14 * np.abs(ra).max()
    I2, K2 = np.meshgrid(np.arange(1, nx + 1), np.arange(1, nz + 1), indexing="ij")
    for s, jr in ((0, 0), (1, ny + 1)):
        aw = np.where(ident[:, jr, :], 0.0, Ax[unk(I2, np.full_like(I2, jr), K2)])
        rr = np.where(ident[:, jr, :], 0.0, rw[:, s, :])
        assert np.abs(np.abs(rr) - np.abs(aw)).max() <= 1e-14 * np.abs(aw).max()
