"""Walls in x and z (ip = 1, kp = 1) against the oracle.

With walls the ghost cells of that direction hold the value of the wall
relation of mul_boun_sndrcv (multigrid.f03:1111-1158, 1280-1316: the flux
through the wall face equals an*cs/dt) and its edge copies (:1360-1742),
instead of periodic images.  The oracle runs two emulated ranks where z has
walls: on one rank the reference leaves the edge cells of the last plane
unset (multigrid.f03:1628-1742 uses else-if on the rank), so its fixed point
depends on stale values there.

Tolerances: face metric bit-exact; ghost layer at the fixed point of the
fill within 1e-12; solves to ||r||/||b|| <= 1e-10 within 1e-8 of the oracle's
converged solution (zero mean, L2 and max).
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from ples_gb300 import synthetic as S

pytestmark = pytest.mark.gpu
DIMS = (32, 16, 32)
CASES = [(1, 0, 1), (0, 1, 2), (1, 1, 2)]  # ip, kp, oracle ranks


def _zm(fi):
    p = fi[1:-1, 1:-1, 1:-1]
    return p - p.mean()


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b), np.abs(a - b).max() / np.abs(b).max()


@pytest.fixture(scope="module")
def grid():
    return S.wavy_channel_grid(*DIMS, 0.08, 2.0)


@pytest.mark.parametrize("ip,kp,nproc", CASES)
def test_metric_with_walls_bit_exact(grid, ip, kp, nproc):
    from ples_gb300 import mg
    x, y, z = grid
    orc = Oracle(x, y, z, ip=ip, kp=kp, islor=1, nproc=nproc)
    with mg.Multigrid(x, y, z, ip=ip, kp=kp, nlevmax=4) as m:
        for level in (1, 2, 3):
            for name in mg.METRIC_NAMES:
                a, b = m.metric(level, name), orc.metric(level, name)
                assert np.array_equal(a, b), (level, name, np.abs(a - b).max())


def test_wall_ghost_fill_fixed_point(grid):
    """x walls (the oracle's ghost fill runs on one rank; with z walls its
    last-plane edges need the two-rank emulation, covered by the solves)."""
    from ples_gb300 import mg
    x, y, z = grid
    jx, jy, jz = DIMS
    ip, kp = 1, 0
    orc = Oracle(x, y, z, ip=ip, kp=kp, islor=1, dt=0.5)
    rng = np.random.default_rng(5)
    shapes = ((jy, jz), (jy, jz), (jx, jz), (jx, jz), (jx, jy), (jx, jy))
    cs = [np.asfortranarray(0.3 * rng.standard_normal(s)) for s in shapes]
    with mg.Multigrid(x, y, z, ip=ip, kp=kp, nlevmax=4, dt=0.5) as m:
        for level in (1, 2):
            nx, ny, nz = orc.dims(level)
            pr = np.asfortranarray(rng.standard_normal((nx + 2, ny + 2, nz + 2)))
            ref = pr.copy(order="F")
            for _ in range(40):
                ref = orc.ghost_fill(level, ref, cs=cs)
            out = m.ghost_fill(level, pr, cs=cs, passes=200)
            np.testing.assert_array_equal(out[1:-1, 1:-1, 1:-1], pr[1:-1, 1:-1, 1:-1])
            assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max(), (level, np.abs(out - ref).max())


@pytest.mark.parametrize("ip,kp,nproc", CASES)
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_solve_with_walls_matches_oracle(grid, ip, kp, nproc, precision):
    from ples_gb300 import mg
    x, y, z = grid
    rhs = S.divergence_rhs(*DIMS, seed=4)
    fo, *_ = Oracle(x, y, z, ip=ip, kp=kp, islor=1, nproc=nproc).multi(rhs, eps=1e-13, ficycle=600)
    with mg.Multigrid(x, y, z, ip=ip, kp=kp, precision=precision) as m:
        fi, st = m.solve(rhs, rel_tol=1e-10)
    assert st["status"] == mg.OK and st["rel_residual"] <= 1e-10
    l2, mx = _rel(_zm(fi), _zm(fo))
    assert l2 <= 1e-8 and mx <= 1e-8, (l2, mx)


def test_wall_fluxes_on_x_and_z_walls(grid):
    """cs1, cs2 (x walls) and cs5, cs6 (z walls) at dt = 0.5 with the
    right-hand side made compatible with their net flux."""
    from ples_gb300 import mg
    x, y, z = grid
    jx, jy, jz = DIMS
    dt = 0.5
    rng = np.random.default_rng(12)
    cs = [np.asfortranarray(0.1 * rng.standard_normal(s))
          for s in ((jy, jz), (jy, jz), (jx, jz), (jx, jz), (jx, jy), (jx, jy))]
    net = ((cs[1].sum() - cs[0].sum()) + (cs[3].sum() - cs[2].sum()) + (cs[5].sum() - cs[4].sum())) / dt
    rhs = S.divergence_rhs(*DIMS, seed=8, dt=dt)
    rhs = rhs + net / rhs.size
    orc = Oracle(x, y, z, ip=1, kp=1, islor=1, nproc=2, dt=dt)
    fo, *_ = orc.multi(rhs, cs=cs, eps=1e-13, ficycle=600)
    with mg.Multigrid(x, y, z, ip=1, kp=1, dt=dt) as m:
        fi, st = m.solve(rhs, cs=cs, rel_tol=1e-10)
    assert st["status"] == mg.OK and abs(st["rhs_mean_removed"]) < 1e-12
    l2, mx = _rel(_zm(fi), _zm(fo))
    assert l2 <= 1e-8 and mx <= 1e-8, (l2, mx)


def test_walls_in_a_batch_and_rejected_with_a_mask(grid):
    """A walled member of a batch is solved by the single-grid solver within
    the batch call (the same field as its own solve); walls and an
    immersed-boundary mask together are rejected at creation."""
    from ples_gb300 import mg
    x, y, z = grid
    rhs = S.divergence_rhs(*DIMS, seed=9)
    with mg.Multigrid(x, y, z, ip=1) as m:
        fs, ss = m.solve(rhs, rel_tol=1e-10)
        with mg.Batch([m]) as b:
            (fb,), (sb,) = b.solve([rhs], rel_tol=1e-10)
    assert ss["status"] == mg.OK and sb["status"] == mg.OK
    np.testing.assert_array_equal(fb, fs)
    with pytest.raises(mg.PlesMGError):
        mg.Multigrid(x, y, z, kp=1, solid=np.zeros(DIMS, dtype=bool))


def _step_inputs_walls(ip, kp, seed):
    """Intermediate Cartesian velocities with wall velocities in the ghost
    cells of walled directions and images in periodic ones; previous
    contravariant velocities whose wall faces carry mean-zero old fluxes."""
    jx, jy, jz = DIMS
    rng = np.random.default_rng(seed)
    u, v, w = (rng.standard_normal((jx + 2, jy + 2, jz + 2)) for _ in range(3))
    for a in (u, v, w):
        if ip == 0:
            a[0], a[jx + 1] = a[jx], a[1]
        if kp == 0:
            a[:, :, 0], a[:, :, jz + 1] = a[:, :, jz], a[:, :, 1]
    uc = rng.standard_normal((jx + 1, jy, jz))
    vc = rng.standard_normal((jx, jy + 1, jz))
    wc = rng.standard_normal((jx, jy, jz + 1))
    for f in (0, jy):
        vc[:, f] -= vc[:, f].mean()
    if ip:
        for f in (0, jx):
            uc[f] -= uc[f].mean()
    if kp:
        for f in (0, jz):
            wc[:, :, f] -= wc[:, :, f].mean()
    return u, v, w, uc, vc, wc


@pytest.mark.parametrize("ip,kp,nproc", CASES)
def test_pressure_step_with_walls_matches_oracle(grid, ip, kp, nproc):
    """ples_mg_step with x/z walls: contra's wall fluxes cs1/cs2/cs5/cs6 on
    the device, the solve, and vel_up leaving the wall faces alone, against
    the oracle chain (to 1e-8 for the pressure, 1e-12 for the velocities);
    the result is divergence free against the old wall fluxes."""
    from oracle.projection import contra_walls, diver, project
    from ples_gb300 import mg
    x, y, z = grid
    jx, jy, jz = DIMS
    dt = 0.01
    u, v, w, uc, vc, wc = _step_inputs_walls(ip, kp, 50 + ip + 2 * kp)
    orc = Oracle(x, y, z, ip=ip, kp=kp, islor=1, dt=dt, nproc=nproc)
    uc1, vc1, wc1, cs = contra_walls(orc, u, v, w, uc, vc, wc)
    with mg.Multigrid(x, y, z, ip=ip, kp=kp, dt=dt) as m:
        (u2, v2, w2, uc2, vc2, wc2, fi), st = m.step(u, v, w, uc, vc, wc, np.zeros((jx + 2, jy + 2, jz + 2)),
                                                     rel_tol=1e-10)
    assert st["status"] == mg.OK and abs(st["rhs_mean_removed"]) < 1e-9
    ref, *_ = orc.multi(diver(uc1, vc1, wc1, dt), cs=cs, eps=1e-13, ficycle=800)
    l2, mx = _rel(_zm(fi), _zm(ref))
    assert l2 <= 1e-8 and mx <= 1e-8, (l2, mx)
    exp = project(orc, fi, uc1, vc1, wc1, u, v, w, dt)
    for got, want in zip((uc2, vc2, wc2, u2, v2, w2), exp):
        assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    old = [uc2.copy(), vc2.copy(), wc2.copy()]
    old[1][:, 0], old[1][:, jy] = vc[:, 0], vc[:, jy]
    if ip:
        old[0][0], old[0][jx] = uc[0], uc[jx]
    if kp:
        old[2][:, :, 0], old[2][:, :, jz] = wc[:, :, 0], wc[:, :, jz]
    d0 = np.abs(diver(uc1, vc1, wc1, 1.0)).max()
    assert np.abs(diver(*old, 1.0)).max() <= 1e-8 * d0


def test_steep_wall_grid_never_returns_garbage():
    """x walls on a strongly sheared grid (wall amplitude 0.1, stretching 2.5,
    the benchmark channel's shape): the wall ghost relation is not
    contractive there (2(|g12|+|g13|)/(4 g11) > 2 near the bottom wall) and
    the reference's own solver diverges (the oracle's residual grows by many
    orders in its first cycles).  The device either reports DIVERGED or
    returns a field that satisfies the reference's discrete system."""
    from ples_gb300 import mg
    x, y, z = S.wavy_channel_grid(32, 16, 32, 0.1, 2.5)
    rhs = S.divergence_rhs(32, 16, 32, seed=1)
    orc = Oracle(x, y, z, ip=1, kp=0, islor=1)
    *_, rr = orc.multi(rhs, eps=1e-13, ficycle=3)
    assert not (rr < 1.0)
    with mg.Multigrid(x, y, z, ip=1) as m:
        try:
            fi, st = m.solve(rhs, rel_tol=1e-10)
        except mg.PlesMGError as e:
            assert e.value.code == mg.DIVERGED
        else:
            assert st["status"] == mg.OK
            r, _ = orc.true_residual(fi, rhs - rhs.mean(), passes=3)
            assert np.linalg.norm(r) / np.linalg.norm(rhs) <= 1e-8
        fi, st = m.solve(np.zeros((32, 16, 32), order="F"), rel_tol=1e-10)
        assert st["status"] == mg.OK


def test_divergent_wall_case_is_reported():
    """x and z walls on a wavy, strongly stretched channel: the reference's
    iteration itself ends in NaN there (tests/test_oracle.py); the device
    solve stops with PLES_MG_DIVERGED rather than returning a field."""
    from ples_gb300 import mg
    dims = (64, 32, 64)
    x, y, z = S.wavy_channel_grid(*dims, 0.1, 2.5)
    rhs = S.divergence_rhs(*dims, seed=4)
    with mg.Multigrid(x, y, z, ip=1, kp=1) as m:
        with pytest.raises(mg.PlesMGError) as e:
            m.solve(rhs, rel_tol=1e-10, max_cycles=40)
    assert e.value.code == mg.DIVERGED
