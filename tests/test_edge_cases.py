"""Edge cases of the solve through the C ABI: the smallest grids the ABI
accepts and odd-sized ones against the oracle (converged solutions within
1e-8, zero mean), a zero right-hand side, max_cycles = 0, non-finite input
(reported as DIVERGED, the handle stays usable), and repeated solves on one
handle with changing right-hand sides (the captured outer-iteration graph is
reused) agreeing with fresh handles bit for bit.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from ples_gb300 import synthetic as S

pytestmark = pytest.mark.gpu
SOL_TOL = 1e-8


def _zm(fi):
    p = fi[1:-1, 1:-1, 1:-1]
    return p - p.mean()


@pytest.mark.parametrize("dims", [(8, 4, 8), (10, 6, 12)])
def test_smallest_grids_match_oracle(dims):
    from ples_gb300 import mg
    x, y, z = S.wavy_channel_grid(*dims, 0.05, 1.5)
    rhs = S.divergence_rhs(*dims, seed=5)
    fo, *_ = Oracle(x, y, z, islor=1).multi(rhs, eps=1e-13, ficycle=400)
    for prec in ("mixed", "fp64"):
        with mg.Multigrid(x, y, z, precision=prec) as m:
            fi, st = m.solve(rhs, rel_tol=1e-10)
        assert st["status"] == mg.OK
        a, b = _zm(fi), _zm(fo)
        assert np.linalg.norm(a - b) / np.linalg.norm(b) <= SOL_TOL
        assert np.abs(a - b).max() / np.abs(b).max() <= SOL_TOL


def test_zero_rhs_and_no_cycles():
    from ples_gb300 import mg
    dims = (16, 8, 16)
    x, y, z = S.wavy_channel_grid(*dims, 0.05, 1.5)
    with mg.Multigrid(x, y, z) as m:
        fi, st = m.solve(np.zeros(dims, order="F"), rel_tol=1e-10)
        assert st["status"] == mg.OK and st["outer_iterations"] == 0 and st["vcycles"] == 0
        assert not fi.any()
        rhs = S.divergence_rhs(*dims, seed=6)
        fi, st = m.solve(rhs, rel_tol=1e-10, max_cycles=0)
        assert st["status"] == mg.NOT_CONVERGED and st["vcycles"] == 0
        assert st["rel_residual"] == pytest.approx(1.0, rel=1e-12)


def test_non_finite_input_reports_diverged_and_handle_recovers():
    from ples_gb300 import mg
    dims = (16, 8, 16)
    x, y, z = S.wavy_channel_grid(*dims, 0.05, 1.5)
    rhs = S.divergence_rhs(*dims, seed=7)
    with mg.Multigrid(x, y, z) as m:
        ref, _ = m.solve(rhs, rel_tol=1e-10)
        bad = rhs.copy(order="F")
        bad[3, 2, 5] = np.nan
        with pytest.raises(mg.PlesMGError) as e:
            m.solve(bad, rel_tol=1e-10)
        assert e.value.code == mg.DIVERGED
        fi0 = np.zeros((dims[0] + 2, dims[1] + 2, dims[2] + 2), order="F")
        fi0[4, 4, 4] = np.inf
        with pytest.raises(mg.PlesMGError) as e:
            m.solve(rhs, fi=fi0, rel_tol=1e-10)
        assert e.value.code == mg.DIVERGED
        again, st = m.solve(rhs, rel_tol=1e-10)
        assert st["status"] == mg.OK and np.array_equal(again, ref)


def test_repeated_solves_reuse_the_graph():
    from ples_gb300 import mg
    dims = (32, 16, 32)
    x, y, z = S.wavy_channel_grid(*dims, 0.08, 2.0)
    rhss = [S.divergence_rhs(*dims, seed=s) for s in (11, 12, 13)]
    with mg.Multigrid(x, y, z) as m:
        seq = [m.solve(r, rel_tol=1e-10)[0] for r in rhss + rhss[:1]]
    assert np.array_equal(seq[0], seq[3])
    for r, f in zip(rhss, seq):
        with mg.Multigrid(x, y, z) as fresh:
            assert np.array_equal(fresh.solve(r, rel_tol=1e-10)[0], f)
