"""A seeded sweep of small problems against the oracle, through the C ABI.

Each case draws its size, wall amplitude and stretching, walls in x and z,
the smoother (zebra line SOR, eta-line Jacobi, zebra with TMA-staged rows,
or the multicolour point SOR with or without a free surface), the
precision, the level count and full or semi-coarsening.  The device solve to
||r||/||b|| <= 1e-12 agrees with the oracle's converged solution (eps 1e-13)
within 1e-8 in the L2 and max norms: of the zero-mean fields, or of the
fields themselves with a free surface (which fixes the pressure level).
Walls and the point smoother are drawn only on mildly sheared grids, where
the reference's own iteration converges (with stronger shear x walls make
it diverge: tests/test_oracle.py).  The oracle runs two emulated ranks when
z has walls, as tests/test_walls.py explains.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from ples_gb300 import mg
from ples_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

SOL_TOL = 1e-8
SIZES = [(32, 16, 32), (48, 32, 48), (64, 32, 32), (32, 32, 64), (40, 16, 24), (24, 8, 16)]


def _draw(seed):
    rng = np.random.default_rng(7000 + seed)
    dims = SIZES[rng.integers(len(SIZES))]
    walls = rng.random() < 0.4
    point = not walls and rng.random() < 0.35
    mild = walls or point
    # the line smoother's other forms: eta-line Jacobi, rows staged by TMA
    # (FP32, periodic); semi-coarsening of the hierarchy
    other = 0 if point else int(rng.choice([0, 0, 0, 1, 2]))
    coarsening = int(rng.random() < 0.3)
    amp = float(rng.uniform(0.0, 0.05 if mild else 0.12))
    beta = float(rng.uniform(1.2, 1.8 if mild else 2.6))
    ip = kp = 0
    if walls:
        ip = int(rng.random() < 0.6)
        # z walls need two oracle ranks, whose planes must split evenly on
        # the oracle's four levels
        kp = int((not ip or rng.random() < 0.5) and dims[2] % 16 == 0)
        if not ip and not kp:
            ip = 1
    fs = point and rng.random() < 0.5
    precision = ("mixed", "fp64")[int(rng.integers(2))]
    if other == 2:  # the TMA-staged rows are FP32 and periodic only
        other, precision = (0, precision) if walls else (2, "mixed")
    return dict(dims=dims, amp=amp, beta=beta, ip=ip, kp=kp, smoother=3 if point else other, fs=fs,
                precision=precision, nlevmax=(0, 4)[int(rng.integers(2))], coarsening=coarsening,
                seed=int(rng.integers(1 << 30)))


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b), np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("case", range(24))
def test_random_problem_against_the_oracle(case):
    c = _draw(case)
    jx, jy, jz = c["dims"]
    x, y, z = S.wavy_channel_grid(jx, jy, jz, c["amp"], c["beta"])
    rhs = S.divergence_rhs(jx, jy, jz, seed=c["seed"])
    orc = Oracle(x, y, z, ip=c["ip"], kp=c["kp"], islor=0 if c["smoother"] == 3 else 1,
                 omega=1.0 if c["smoother"] == 3 else 1.6, nproc=2 if c["kp"] else 1)
    prs = None
    if c["fs"]:
        rng = np.random.default_rng(c["seed"])
        prs = np.asfortranarray(0.1 * rng.standard_normal((jx, jz)))
        orc.set_free_surface(True, prs)
    fo, _, _, rr = orc.multi(rhs, eps=1e-13, ficycle=3000)
    assert rr <= 1e-13, (c, rr)
    kw = dict(ip=c["ip"], kp=c["kp"], precision=c["precision"], smoother=c["smoother"], nlevmax=c["nlevmax"],
              coarsening=c["coarsening"])
    if c["fs"]:
        kw["freesurface"] = 1
    with mg.Multigrid(x, y, z, **kw) as m:
        if c["fs"]:
            m.set_surface_pressure(prs)
        fi, st = m.solve(rhs, rel_tol=1e-12, max_cycles=400)
    assert st["status"] == mg.OK, (c, st)
    a, b = fi[1:-1, 1:-1, 1:-1], fo[1:-1, 1:-1, 1:-1]
    if not c["fs"]:  # the pressure level is free: compare zero-mean fields
        a, b = a - a.mean(), b - b.mean()
    l2, mx = _rel(a, b)
    assert l2 <= SOL_TOL and mx <= SOL_TOL, (c, l2, mx)
