"""Batched solves and the request server, through the C ABI.

Tolerances: every member converged to ||r||/||b|| <= 1e-10; zero-mean
solutions within 1e-8 (L2 and max, relative) of the oracle's converged
solution, and within 1e-9 of the same grid solved alone by ples_mg_solve
(same kernels; only the reduction order of the compatibility shift
differs).  A request's result is the same alone and in a mix of concurrent
requests (each member's arithmetic is independent of the others): within
1e-12.
"""
import threading

import numpy as np
import pytest

from oracle.oracle import Oracle
from ples_gb300 import mg
from ples_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10


def _zm(fi):
    p = fi[1:-1, 1:-1, 1:-1]
    return p - p.mean()


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b), np.abs(a - b).max() / np.abs(b).max()


# uneven sizes and depths (coarsest 3x2x3 .. 4x2x4, 4 to 6 levels)
SIZES = [(32, 16, 32), (48, 32, 48), (24, 16, 24), (64, 32, 64), (32, 32, 32)]


def _case(dims, seed):
    rng = np.random.default_rng(seed)
    amp, beta = rng.uniform(0.0, 0.15), rng.uniform(1.5, 3.0)
    x, y, z = S.wavy_channel_grid(*dims, amp, beta)
    return x, y, z, S.divergence_rhs(*dims, seed=seed)


@pytest.fixture(scope="module")
def cases():
    return [_case(d, 100 + i) for i, d in enumerate(SIZES)]


def test_batch_matches_single_solves_and_oracle(cases):
    members = [mg.Multigrid(x, y, z) for x, y, z, _ in cases]
    rhs = [c[3] for c in cases]
    with mg.Batch(members) as b:
        fis, sts = b.solve(rhs, rel_tol=REL_TOL)
        info = b.info()
        assert info["steps"] > 50
        # again, from zero: identical (the same graph, deterministic)
        fis2, sts2 = b.solve(rhs, rel_tol=REL_TOL)
    for i, (fi, st) in enumerate(zip(fis, sts)):
        assert st["status"] == mg.OK and st["rel_residual"] <= REL_TOL, (i, st)
        np.testing.assert_array_equal(fi, fis2[i])
        assert sts2[i]["outer_iterations"] == st["outer_iterations"]
        fo, so = members[i].solve(rhs[i], rel_tol=REL_TOL)
        l2, mx = _rel(_zm(fi), _zm(fo))
        assert l2 <= 1e-9 and mx <= 1e-9, (i, l2, mx)
        assert abs(st["outer_iterations"] - so["outer_iterations"]) <= 1
    # the oracle on the smallest member
    x, y, z, r = cases[2]
    ref, *_ = Oracle(x, y, z, islor=1).multi(r, eps=1e-13, ficycle=400)
    l2, mx = _rel(_zm(fis[2]), _zm(ref))
    assert l2 <= 1e-8 and mx <= 1e-8
    for m in members:
        m.close()


def test_batch_with_members_outside_the_step_list(cases):
    """FP64, x-walled and point-SOR members join a batch with a plain one:
    the step list covers the plain member and the others are solved one
    after another by the single-grid solver within the same call, so their
    fields are the ones a single solve gives, bit for bit, and the plain
    member's agrees with its single solve within 1e-9."""
    x, y, z, rhs = cases[0]
    xw, yw, zw = S.wavy_channel_grid(32, 16, 32, 0.05, 2.0)  # walls need a grid whose x relation contracts
    rw = S.divergence_rhs(32, 16, 32, seed=61)
    xp, yp, zp = S.wavy_channel_grid(32, 16, 32, 0.03, 1.3)  # mild stretching for the point smoother
    rp = S.divergence_rhs(32, 16, 32, seed=62)
    members = [mg.Multigrid(x, y, z), mg.Multigrid(x, y, z, precision="fp64"), mg.Multigrid(xw, yw, zw, ip=1),
               mg.Multigrid(xp, yp, zp, smoother=3)]
    rhs_l = [rhs, rhs, rw, rp]
    try:
        singles = [m.solve(r, rel_tol=REL_TOL) for m, r in zip(members, rhs_l)]
        with mg.Batch(members) as b:
            fis, sts = b.solve(rhs_l, rel_tol=REL_TOL)
        for i, ((fs, ss), fb, sb) in enumerate(zip(singles, fis, sts)):
            assert sb["status"] == mg.OK and sb["rel_residual"] <= REL_TOL, (i, sb)
            if i == 0:
                assert np.abs(fb - fs).max() <= 1e-9 * np.abs(fs).max()
            else:
                np.testing.assert_array_equal(fb, fs)
                assert sb["outer_iterations"] == ss["outer_iterations"]
        # the server takes them too: a request to the walled member (warm
        # start from its last solution) gives its single solve
        with mg.Server(members[:3]) as s:
            fo, so = s.wait(s.submit(2, rw, rel_tol=REL_TOL))
        assert so["status"] == mg.OK
        assert np.abs(fo - singles[2][0]).max() <= 1e-9 * np.abs(singles[2][0]).max()
    finally:
        for m in members:
            m.close()


def test_batch_with_masked_and_typed_members():
    """Members with an immersed-boundary mask and with PLES cell types in one
    batch with a plain member: each batched result agrees with the same grid
    solved alone within 1e-9 (the sums of the compatibility shift and the
    mean are reduced in another order), the masked member's field vanishes
    on its solid cells and the typed member's max residual is its fluid-cell
    stop test (within 1e-2 of the single solve's: both are FP64 residuals of
    ~1e-11 of slightly different converged fields)."""
    dims = (32, 16, 32)
    x, y, z = S.wavy_channel_grid(*dims, 0.08, 2.0)
    solid = S.sphere_mask(x, y, z, n=6, rmin=0.3, rmax=0.5, seed=3)
    tipo = np.full((dims[0] + 2, dims[1] + 2, dims[2] + 2), 2, dtype=np.int32, order="F")
    tipo[8:14, 4:9, 10:18] = 0
    rhs = [S.divergence_rhs(*dims, seed=s) for s in (41, 42, 43)]
    opts = [dict(solid=solid), dict(tipo=tipo), {}]
    members = [mg.Multigrid(x, y, z, **o) for o in opts]
    try:
        singles = [m.solve(r, rel_tol=REL_TOL) for m, r in zip(members, rhs)]
        with mg.Batch(members) as b:
            fis, sts = b.solve(rhs, rel_tol=REL_TOL)
        for (fs, ss), fb, sb in zip(singles, fis, sts):
            assert sb["status"] == mg.OK and ss["status"] == mg.OK and sb["rel_residual"] <= REL_TOL
            assert np.abs(fb - fs).max() <= 1e-9 * np.abs(fs).max()
        assert np.all(fis[0][1:-1, 1:-1, 1:-1][solid] == 0.0)
        assert sts[1]["max_residual"] == pytest.approx(singles[1][1]["max_residual"], rel=1e-2)
    finally:
        for m in members:
            m.close()


def test_server_same_result_alone_and_in_the_mix(cases):
    # identical grids on separate handles, both starting from zero
    alone = [mg.Multigrid(*cases[1][:3])]
    mix = [mg.Multigrid(*c[:3]) for c in cases[:4]]
    with mg.Server(alone) as s:
        r1, st1 = s.wait(s.submit(0, cases[1][3], rel_tol=REL_TOL))
    assert st1["status"] == mg.OK and st1["rel_residual"] <= REL_TOL
    with mg.Server(mix, hbm_budget_bytes=150e9) as s:
        tickets = {}
        lock = threading.Lock()

        def client(i):
            t = s.submit(i, cases[i][3], rel_tol=REL_TOL)
            with lock:
                tickets[i] = t

        th = [threading.Thread(target=client, args=(i,)) for i in (0, 2, 3, 1)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        res = {i: s.wait(tickets[i]) for i in tickets}
        rep = s.report()
    r2, st2 = res[1]
    assert st2["status"] == mg.OK
    assert np.abs(r2 - r1).max() <= 1e-12 * np.abs(r1).max()
    assert st2["outer_iterations"] == st1["outer_iterations"]
    assert rep["completed"] == 4 and rep["p99_ms"] >= rep["p50_ms"] > 0.0
    for i, (fi, st) in res.items():
        assert st["status"] == mg.OK and st["rel_residual"] <= REL_TOL
    for m in alone + mix:
        m.close()


def test_server_warm_start_and_budget(cases):
    x, y, z, rhs = cases[0]
    with mg.Multigrid(x, y, z) as m:
        with pytest.raises(mg.PlesMGError):
            mg.Server([m], hbm_budget_bytes=1e3)
        with mg.Server([m]) as s:
            _, cold = s.wait(s.submit(0, rhs, rel_tol=REL_TOL))
            rng = np.random.default_rng(5)
            # a small change of the right-hand side: the warm start begins
            # some eight decades closer to the new solution
            rhs2 = rhs + 1e-8 * rng.standard_normal(rhs.shape)
            rhs2 -= rhs2.mean()
            fi, warm = s.wait(s.submit(0, rhs2, rel_tol=REL_TOL))
        assert warm["status"] == mg.OK
        assert warm["outer_iterations"] < cold["outer_iterations"]
        fo, _ = m.solve(rhs2, rel_tol=REL_TOL)
        l2, mx = _rel(_zm(fi), _zm(fo))
        assert l2 <= 1e-8 and mx <= 1e-8


def test_server_queued_requests_match_one_at_a_time(cases):
    """Three requests queued at once for one member, beside a request for
    another: the server stages the next right-hand side while the current
    request solves and admits it as soon as that one finishes.  Each result
    is the one the same requests give submitted one after another (each
    warm-started from the solution before it), within 1e-12."""
    x, y, z, rhs = cases[0]
    other = cases[1]
    rng = np.random.default_rng(11)
    rhss = []
    for _ in range(3):
        r = rhs + 0.05 * np.abs(rhs).max() * rng.standard_normal(rhs.shape)
        rhss.append(r - r.mean())
    with mg.Multigrid(x, y, z) as m, mg.Multigrid(*other[:3]) as m2:
        with mg.Server([m, m2]) as s:
            seq = [s.wait(s.submit(0, r, rel_tol=REL_TOL)) for r in rhss]
    with mg.Multigrid(x, y, z) as m, mg.Multigrid(*other[:3]) as m2:
        with mg.Server([m, m2]) as s:
            t_other = s.submit(1, other[3], rel_tol=REL_TOL)
            tickets = [s.submit(0, r, rel_tol=REL_TOL) for r in rhss]
            queued = [s.wait(t) for t in tickets]
            _, st_other = s.wait(t_other)
            rep = s.report()
    assert st_other["status"] == mg.OK and rep["completed"] == 4
    for (fa, sa), (fb, sb) in zip(seq, queued, strict=True):
        assert sa["status"] == sb["status"] == mg.OK
        assert sa["outer_iterations"] == sb["outer_iterations"]
        assert np.abs(fb - fa).max() <= 1e-12 * np.abs(fa).max()
    # the later requests started warm: no more outer iterations than the first
    assert seq[2][1]["outer_iterations"] <= seq[0][1]["outer_iterations"]


def test_autotune_then_batch(cases):
    """Tuned settings stay in their candidate sets, the tuned single-grid
    solve still converges to the oracle's solution, and a batch of tuned
    members (different sweep counts and smoother widths) matches them."""
    sub = cases[:3]
    members = [mg.Multigrid(*c[:3]) for c in sub]
    tuned = [m.autotune(c[3]) for m, c in zip(members, sub)]
    for t in tuned:
        assert t["nu_pre"] in (1, 2, 3) and t["nu_post"] in (1, 2, 3) and t["inner_cycles"] in (2, 3, 4, 5, 6, 8)
        assert (t["nu_pre"] + t["nu_post"]) * t["inner_cycles"] % 2 == 0 and t["omega"] in (1.3, 1.4)
        assert set(t["line_threads"]) <= {128, 256, 512, 1024} and t["candidates"] >= 13
    with mg.Batch(members) as b:
        fis, sts = b.solve([c[3] for c in sub], rel_tol=REL_TOL)
    for m, c, fi, st in zip(members, sub, fis, sts):
        assert st["status"] == mg.OK and st["rel_residual"] <= REL_TOL
        fo, so = m.solve(c[3], rel_tol=REL_TOL)
        assert so["status"] == mg.OK
        l2, mx = _rel(_zm(fi), _zm(fo))
        assert l2 <= 1e-9 and mx <= 1e-9
    x, y, z, r = sub[2]
    ref, *_ = Oracle(x, y, z, islor=1).multi(r, eps=1e-13, ficycle=400)
    l2, mx = _rel(_zm(fis[2]), _zm(ref))
    assert l2 <= 1e-8 and mx <= 1e-8
    for m in members:
        m.close()
