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
