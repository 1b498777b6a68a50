"""The creation probe of the zebra smoother's default settings.

The fast defaults (one sweep before and two after the coarse correction,
six V-cycles per outer iteration, omega 1.4) diverge on some strongly
stretched small grids; a handle created with all of omega, nu_pre, nu_post
and inner_cycles left at 0 solves a pseudo-random right-hand side for two
outer iterations and, if that does not converge, takes two sweeps each
side, five V-cycles and omega 1.3.  The settings a handle took show in its
solves: V-cycles = outer iterations x V-cycles per outer iteration.  The
grid below is the 24x8x16 channel stretched at 2.36 that the seeded parity
sweep found.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from ples_gb300 import mg
from ples_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

DIMS = (24, 8, 16)
AMP, BETA, SEED = 0.04351888113605135, 2.3558716851288906, 417409219


def _solve_ok(m, rhs):
    try:
        fi, st = m.solve(rhs, rel_tol=1e-12, max_cycles=400)
    except mg.PlesMGError:  # diverged
        return None, None
    return (fi, st) if st["status"] == mg.OK else (None, st)


def test_probe_falls_back_where_the_fast_defaults_diverge():
    x, y, z = S.wavy_channel_grid(*DIMS, AMP, BETA)
    rhs = S.divergence_rhs(*DIMS, seed=SEED)
    # the fast settings given explicitly: no probe, no convergence
    with mg.Multigrid(x, y, z, precision="fp64", nlevmax=4, omega=1.4, nu_pre=1, nu_post=2,
                      inner_cycles=6) as m:
        fi, _ = _solve_ok(m, rhs)
    assert fi is None
    # the defaults: the probe takes the earlier settings, five V-cycles per
    # outer iteration, and the solve matches the oracle
    with mg.Multigrid(x, y, z, precision="fp64", nlevmax=4) as m:
        fi, st = _solve_ok(m, rhs)
    assert fi is not None, st
    assert st["vcycles"] == 5 * st["outer_iterations"]
    fo, _, _, rr = Oracle(x, y, z, islor=1).multi(rhs, eps=1e-13, ficycle=3000)
    assert rr <= 1e-13
    a, b = fi[1:-1, 1:-1, 1:-1], fo[1:-1, 1:-1, 1:-1]
    a, b = a - a.mean(), b - b.mean()
    assert np.linalg.norm(a - b) <= 1e-8 * np.linalg.norm(b)


def test_probe_keeps_the_fast_defaults_on_a_mild_grid():
    jx, jy, jz = 32, 16, 32
    x, y, z = S.wavy_channel_grid(jx, jy, jz, 0.05, 2.0)
    rhs = S.divergence_rhs(jx, jy, jz, seed=0)
    for precision in ("mixed", "fp64"):
        with mg.Multigrid(x, y, z, precision=precision) as m:
            fi, st = _solve_ok(m, rhs)
        assert fi is not None, st
        assert st["vcycles"] == 6 * st["outer_iterations"], (precision, st)
