"""Projection step around the solve (diver, multi, gradie, vel_up) through
ples_mg_project, and the whole pressure step with contra in front through
ples_mg_step, against oracle/projection.py.

Tolerances: the restated face normals rebuild the C oracle's g11, g22, g33
to 1e-13 (the pin of the normals); the device's new face and cell
velocities match the oracle's projection of the device pressure to 1e-12
relative; the pressure matches the oracle solver's to 1e-8 (zero mean);
the divergence of the projected face velocities drops to <= 1e-8 of its
value before (the solve stops at ||r||/||b|| <= 1e-10).  The oracle's
contra is pinned by a geometric identity: the face normals of a cell sum to
zero, so a uniform velocity gives zero divergence to round-off (1e-12 of
the face fluxes).
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from oracle.projection import contra, diver, face_normals, project
from ples_gb300 import synthetic as S

DIMS = (32, 16, 32)
DT = 0.01


@pytest.fixture(scope="module")
def case():
    x, y, z = S.wavy_channel_grid(*DIMS, 0.08, 2.0)
    rng = np.random.default_rng(31)
    jx, jy, jz = DIMS
    uc = rng.standard_normal((jx + 1, jy, jz))
    uc[0] = uc[jx]  # periodic faces
    vc = rng.standard_normal((jx, jy + 1, jz))
    vc[:, 0] = vc[:, jy] = 0.0  # no flux through the walls
    wc = rng.standard_normal((jx, jy, jz + 1))
    wc[:, :, 0] = wc[:, :, jz]
    u, v, w = (rng.standard_normal((jx + 2, jy + 2, jz + 2)) for _ in range(3))
    return dict(x=x, y=y, z=z, uc=uc, vc=vc, wc=wc, u=u, v=v, w=w, orc=Oracle(x, y, z, islor=1))


def test_face_normals_rebuild_the_metric(case):
    orc = case["orc"]
    (csx, csy, csz, jc), (etx, ety, etz, je), (ztx, zty, ztz, jz_) = face_normals(orc)
    for got, ref in (((csx ** 2 + csy ** 2 + csz ** 2) / jc, orc.metric(1, "g11")),
                     ((etx ** 2 + ety ** 2 + etz ** 2) / je, orc.metric(1, "g22")),
                     ((ztx ** 2 + zty ** 2 + ztz ** 2) / jz_, orc.metric(1, "g33"))):
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.gpu
def test_device_projection_matches_oracle(case):
    from ples_gb300 import mg
    jx, jy, jz = DIMS
    fi0 = np.zeros((jx + 2, jy + 2, jz + 2))
    with mg.Multigrid(case["x"], case["y"], case["z"], precision="mixed", dt=DT) as m:
        (uc, vc, wc, fi, u, v, w), st = m.project(case["uc"], case["vc"], case["wc"], fi0, case["u"], case["v"],
                                                  case["w"], rel_tol=1e-10)
    assert st["status"] == mg.OK and st["rel_residual"] <= 1e-10
    # the pressure: the oracle solver on the same right-hand side
    rhs = diver(case["uc"], case["vc"], case["wc"], DT)
    ref, *_ = case["orc"].multi(rhs, eps=1e-13, ficycle=400)
    a, b = fi[1:-1, 1:-1, 1:-1], ref[1:-1, 1:-1, 1:-1]
    a, b = a - a.mean(), b - b.mean()
    assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 1e-8
    # the velocity updates of that pressure
    exp = project(case["orc"], fi, case["uc"], case["vc"], case["wc"], case["u"], case["v"], case["w"], DT)
    for got, want in zip((uc, vc, wc, u, v, w), exp):
        assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    # the projected face velocities are divergence free to the solve's tolerance
    d0 = np.abs(diver(case["uc"], case["vc"], case["wc"], 1.0)).max()
    d1 = np.abs(diver(uc, vc, wc, 1.0)).max()
    assert d1 <= 1e-8 * d0, (d1, d0)


def _step_inputs(jx, jy, jz, seed):
    """Intermediate Cartesian velocities with periodic images in x and z and
    a moving-wall velocity in the ghost rows, and previous contravariant
    velocities whose wall faces carry net-zero old wall fluxes."""
    rng = np.random.default_rng(seed)
    u, v, w = (rng.standard_normal((jx + 2, jy + 2, jz + 2)) for _ in range(3))
    for a in (u, v, w):
        a[0], a[jx + 1] = a[jx], a[1]
        a[:, :, 0], a[:, :, jz + 1] = a[:, :, jz], a[:, :, 1]
    uc = rng.standard_normal((jx + 1, jy, jz))
    vc = rng.standard_normal((jx, jy + 1, jz))
    wc = rng.standard_normal((jx, jy, jz + 1))
    for jf in (0, jy):
        vc[:, jf] -= vc[:, jf].mean()
    return u, v, w, uc, vc, wc


def test_oracle_contra_uniform_flow_is_divergence_free(case):
    jx, jy, jz = DIMS
    orc = case["orc"]
    u = np.full((jx + 2, jy + 2, jz + 2), 0.7)
    v = np.full_like(u, -0.3)
    w = np.full_like(u, 1.1)
    vc_old = np.zeros((jx, jy + 1, jz))
    uc, vc, wc, cs3, cs4 = contra(orc, u, v, w, vc_old)
    scale = max(np.abs(uc).max(), np.abs(vc).max(), np.abs(wc).max())
    assert np.abs(diver(uc, vc, wc, 1.0)).max() <= 1e-12 * scale
    assert np.array_equal(cs3, vc[:, 0]) and np.array_equal(cs4, vc[:, jy])


@pytest.mark.gpu
def test_device_step_matches_oracle(case):
    """ples_mg_step = contra, then the projection: the pressure matches the
    oracle solver on the oracle's contra right-hand side and wall fluxes,
    the velocities match the oracle's projection of the device pressure."""
    from ples_gb300 import mg
    jx, jy, jz = DIMS
    u, v, w, uc, vc, wc = _step_inputs(jx, jy, jz, 41)
    orc = Oracle(case["x"], case["y"], case["z"], islor=1, dt=DT)
    uc1, vc1, wc1, cs3, cs4 = contra(orc, u, v, w, vc)
    assert np.abs(cs3).max() > 0.1 and np.abs(cs4).max() > 0.1
    fi0 = np.zeros((jx + 2, jy + 2, jz + 2))
    with mg.Multigrid(case["x"], case["y"], case["z"], precision="mixed", dt=DT) as m:
        (u2, v2, w2, uc2, vc2, wc2, fi), st = m.step(u, v, w, uc, vc, wc, fi0, rel_tol=1e-10)
    assert st["status"] == mg.OK and st["rel_residual"] <= 1e-10
    rhs = diver(uc1, vc1, wc1, DT)
    zero = np.zeros
    cs = [zero((jy, jz)), zero((jy, jz)), cs3, cs4, zero((jx, jy)), zero((jx, jy))]
    ref, *_ = orc.multi(rhs, cs=cs, eps=1e-13, ficycle=400)
    a, b = fi[1:-1, 1:-1, 1:-1], ref[1:-1, 1:-1, 1:-1]
    a, b = a - a.mean(), b - b.mean()
    assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 1e-8
    exp = project(orc, fi, uc1, vc1, wc1, u, v, w, DT)
    for got, want in zip((uc2, vc2, wc2, u2, v2, w2), exp):
        assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    # the wall condition of the solve is grad(fi).n = cs/dt, so the new field
    # is divergence free against the OLD wall fluxes: the cells next to the
    # walls keep -cs3 and +cs4 of divergence, the others none
    d0 = np.abs(diver(uc1, vc1, wc1, 1.0)).max()
    vc_old_walls = vc2.copy()
    vc_old_walls[:, 0], vc_old_walls[:, jy] = vc[:, 0], vc[:, jy]
    d1 = np.abs(diver(uc2, vc_old_walls, wc2, 1.0)).max()
    assert d1 <= 1e-8 * d0, (d1, d0)
    d = diver(uc2, vc2, wc2, 1.0)
    assert np.abs(d[:, 0] + cs3).max() <= 1e-8 * d0 and np.abs(d[:, -1] - cs4).max() <= 1e-8 * d0
