"""Parity at the benchmark sizes and on the reference's own deck, through the
C ABI (GPU, slow: each runs the CPU oracle on a grid of the benchmark).

* channel 256x128x256 (wall amplitude 0.1, stretch 2.5, RHS seed 1): the
  device's zero-mean solution against the oracle's, which the restated
  reference solver (line SOR, 4 levels, emulated MPI ranks) converges to
  ||r||/||b|| <= 1e-13.  The device solves to 1e-10 (the benchmark
  setting) and to 1e-12, mixed and FP64; all four agree with the oracle
  within 1e-8 in the L2 and max norms.  (A relative residual bounds the
  solution error only through the operator's conditioning: the reference
  algorithm's own 1e-10 iterate is ~6e-7 away from the converged solution
  at this size; the device's dense coarsest solve leaves much less of the
  error in smooth modes.  The test prints both.)
* the reference's sample deck (gri3dp_in.dat, uniform 32^3) at its own
  settings (Agenerale.in:41-52: point SOR islor = 0, omega 1.6, 4 levels,
  absolute max-norm stop eps = 1e-8), the device with its point SOR
  (smoother 3, omega 1.6) and with its line smoother: both solvers stop
  below eps, and their solutions converged to 1e-13 agree within 1e-8.
* the 64-grid batch of uneven sizes (seeds 2..65): every member of the
  batched solve within 1e-9 of the same grid solved alone, and one member
  of each of three sizes within 1e-8 of the oracle.
* the immersed-boundary channel 512x256x512 (32 seeded spheres): the masked
  restatement of the reference's fine-level system (oracle.masked) gives the
  device solution a relative residual <= 2e-10 and wall-row residuals at the
  same level; at 48x24x48 with the same sphere distribution the device
  solution is within 1e-8 of the masked oracle's exact (sparse direct) one,
  and at 64x32x64 its masked residual is at the same level.
"""
import json
import os

import numpy as np
import pytest

from oracle.oracle import Oracle
from ples_gb300 import mg
from ples_gb300 import synthetic as S

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

SOL_TOL = 1e-8


def _zm(fi):
    p = fi[1:-1, 1:-1, 1:-1]
    return p - p.mean()


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b), np.abs(a - b).max() / np.abs(b).max()


def _ranks(jz, levels=4):
    """Emulated MPI ranks for the oracle: the most host threads that divide
    jz at every one of its levels."""
    n = os.cpu_count() or 1
    for p in range(n, 0, -1):
        if (jz >> (levels - 1)) % p == 0:
            return p
    return 1


def test_channel_256x128x256_against_converged_oracle():
    w = S.WORKLOADS["channel_256x128x256"]
    x, y, z = w.grid()
    rhs = w.rhs()
    orc = Oracle(x, y, z, islor=1, nproc=_ranks(w.jz))
    f10, _, _, r10 = orc.multi(rhs, eps=1e-10, ficycle=400)
    assert r10 <= 1e-10
    fo, _, _, rr = orc.multi(rhs, fi=f10, eps=1e-13, ficycle=400)
    assert rr <= 1e-13
    ref = _zm(fo)
    oracle_gap = max(_rel(_zm(f10), ref))
    found = {"oracle_1e-10_vs_converged": oracle_gap}
    for prec in ("mixed", "fp64"):
        with mg.Multigrid(x, y, z, precision=prec) as m:
            for tol in (1e-10, 1e-12):
                fi, st = m.solve(rhs, rel_tol=tol, max_cycles=100)
                assert st["status"] == mg.OK and st["rel_residual"] <= tol, (prec, tol, st)
                l2, mx = _rel(_zm(fi), ref)
                found[f"{prec}_{tol:g}"] = (l2, mx)
                assert l2 <= SOL_TOL and mx <= SOL_TOL, (prec, tol, found)
    print("channel_256x128x256 solution errors vs the converged oracle:", found)


def _deck():
    d = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "sample_deck.json")))
    xs, ys, zs = (np.array(d[c]) for c in "xyz")
    shp = (xs.size, ys.size, zs.size)
    x = np.asfortranarray(np.broadcast_to(xs[:, None, None], shp))
    y = np.asfortranarray(np.broadcast_to(ys[None, :, None], shp))
    z = np.asfortranarray(np.broadcast_to(zs[None, None, :], shp))
    return d, x, y, z


@pytest.mark.parametrize("smoother", [3, 0], ids=["point_sor", "line_sor"])
def test_sample_deck_at_its_own_settings(smoother):
    d, x, y, z = _deck()
    s = d["solver"]
    jx, jy, jz = d["dims"]
    rhs = S.divergence_rhs(jx, jy, jz, seed=0)
    orc = Oracle(x, y, z, islor=s["islor"], omega=s["omega"], nlevmax=s["nlevmultimax"], nproc=2)
    fo, cyc, rmax, _ = orc.multi(rhs, eps=s["eps"], ficycle=s["ficycle"], stop_mode=0)
    assert rmax < s["eps"] and cyc < s["ficycle"]
    omega = s["omega"] if smoother == 3 else 0.0  # the deck's omega is its point SOR's
    with mg.Multigrid(x, y, z, nlevmax=s["nlevmultimax"], precision="fp64", smoother=smoother, omega=omega) as m:
        fi, st = m.solve(rhs, rel_tol=0.0, abs_tol=s["eps"], max_cycles=s["ficycle"])
        assert st["status"] == mg.OK and st["max_residual"] < s["eps"], st
        # both stopped by the same absolute test: their fields differ by the
        # error a max-norm residual of 1e-8 leaves (uniform 32^3 grid)
        l2, mx = _rel(_zm(fi), _zm(fo))
        assert l2 <= 1e-6 and mx <= 1e-6, (l2, mx)
        fo2, _, _, rr = orc.multi(rhs, fi=fo, eps=1e-13, ficycle=2000)
        assert rr <= 1e-13
        fi2, st2 = m.solve(rhs, rel_tol=1e-13, max_cycles=200)
        assert st2["status"] == mg.OK
        l2, mx = _rel(_zm(fi2), _zm(fo2))
        assert l2 <= SOL_TOL and mx <= SOL_TOL, (l2, mx)


def test_batch_of_64_uneven_grids():
    insts = S.batch_instances()
    assert len(insts) == 64
    grids = [w.grid() for w in insts]
    rhs = [w.rhs() for w in insts]
    members = [mg.Multigrid(*g) for g in grids]
    try:
        with mg.Batch(members) as b:
            fbs, sbs = b.solve(rhs, rel_tol=1e-10)
        for i, (m, r, fb, sb) in enumerate(zip(members, rhs, fbs, sbs)):
            assert sb["status"] == mg.OK and sb["rel_residual"] <= 1e-10, (i, sb)
            fs, ss = m.solve(r, rel_tol=1e-10)
            assert ss["status"] == mg.OK
            l2, mx = _rel(_zm(fb), _zm(fs))
            assert l2 <= 1e-9 and mx <= 1e-9, (insts[i].name, l2, mx)
        # one member of each of three sizes against the oracle
        picked = {}
        for i, w in enumerate(insts):
            key = (w.jx, w.jy, w.jz)
            if key in ((32, 32, 32), (48, 32, 48), (64, 64, 64)) and key not in picked:
                picked[key] = i
        assert len(picked) == 3
        for key, i in picked.items():
            fo, *_ = Oracle(*grids[i], islor=1).multi(rhs[i], eps=1e-13, ficycle=400)
            l2, mx = _rel(_zm(fbs[i]), _zm(fo))
            assert l2 <= SOL_TOL and mx <= SOL_TOL, (insts[i].name, l2, mx)
    finally:
        for m in members:
            m.close()


def test_ib_512x256x512_masked_residual_of_device_solution():
    from oracle import masked as M
    w = S.WORKLOADS["channel_512x256x512"]
    x, y, z = w.grid()
    rhs = w.rhs()
    solid = S.sphere_mask(x, y, z, n=32, rmin=0.05, rmax=0.2, seed=11)
    with mg.Multigrid(x, y, z, precision="mixed", solid=solid) as m:
        fi, st = m.solve(rhs, rel_tol=1e-10, max_cycles=100)
    assert st["status"] == mg.OK and st["rel_residual"] <= 1e-10, st
    assert np.all(fi[1:-1, 1:-1, 1:-1][solid] == 0.0)
    orc = Oracle(x, y, z, islor=1, nlevmax=1)
    r, rw = M.residual(orc, fi, rhs, solid)
    fl = ~solid
    b = np.where(fl, rhs, 0.0)
    b = np.where(fl, b - b[fl].mean(), 0.0)
    bn = np.linalg.norm(b)
    assert np.linalg.norm(r) / bn <= 2e-10
    assert np.linalg.norm(rw) / bn <= 2e-10


def test_ib_48x24x48_sphere_distribution_against_sparse_direct():
    """The benchmark's sphere distribution on a grid the sparse-direct
    oracle factors in about two minutes (the 64x32x64 system takes a quarter
    of an hour: fill-in of the 3-D stencil), plus the masked residual of the
    device solution at 64x32x64."""
    from oracle import masked as M
    for nx, ny, nz in ((48, 24, 48), (64, 32, 64)):
        x, y, z = S.wavy_channel_grid(nx, ny, nz, 0.1, 3.0)
        rhs = S.divergence_rhs(nx, ny, nz, seed=4)
        solid = S.sphere_mask(x, y, z, n=32, rmin=0.05, rmax=0.2, seed=11)
        assert solid.any()
        orc = Oracle(x, y, z, islor=1, nlevmax=1)
        ref = M.solve(orc, rhs, solid) if nx == 48 else None
        fl = ~solid
        for prec in ("mixed", "fp64"):
            with mg.Multigrid(x, y, z, precision=prec, solid=solid) as m:
                fi, st = m.solve(rhs, rel_tol=1e-10)
            assert st["status"] == mg.OK, st
            if ref is not None:
                p = fi[1:-1, 1:-1, 1:-1]
                p = np.where(fl, p - p[fl].mean(), 0.0)
                l2, mx = _rel(p, ref)
                assert l2 <= SOL_TOL and mx <= SOL_TOL, (nx, prec, l2, mx)
            r, rw = M.residual(orc, fi, rhs, solid)
            b = np.where(fl, rhs, 0.0)
            bn = np.linalg.norm(np.where(fl, b - b[fl].mean(), 0.0))
            assert np.linalg.norm(r) / bn <= 2e-10 and np.linalg.norm(rw) / bn <= 2e-10, (nx, prec)
