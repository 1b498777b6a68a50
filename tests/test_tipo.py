"""PLES's cell types (tipo: 0 solid, 1 IB, >= 2 fluid) around the solve:
ples_mg_potenziale_ibm against the loop restatement in oracle/ibm.py
(bit-exact), and the max-norm stop test over fluid cells of multi with
bodyforce = 1.  The operator does not depend on tipo, so a solve with and
without it returns the same field; its max_residual is the oracle residual's
max over the fluid cells (to 1e-2 relative: both are FP64 residuals of a
converged field, ~1e-11 in size, evaluated in different orders).
"""
import numpy as np
import pytest

from oracle.ibm import masked_max, potenziale_ibm
from oracle.oracle import Oracle
from ples_gb300 import synthetic as S

DIMS = (32, 16, 32)


@pytest.fixture(scope="module")
def case():
    jx, jy, jz = DIMS
    x, y, z = S.wavy_channel_grid(jx, jy, jz, 0.08, 2.0)
    rng = np.random.default_rng(77)
    tipo = np.full((jx + 2, jy + 2, jz + 2), 2, dtype=np.int32, order="F")
    # a solid block, its face-neighbour shell IB, plus scattered types
    tipo[8:14, 4:9, 10:18] = 0
    shell = np.zeros_like(tipo, dtype=bool)
    for ax in range(3):
        for s in (1, -1):
            shell |= np.roll(tipo == 0, s, axis=ax)
    tipo[shell & (tipo != 0)] = 1
    pick = rng.random(tipo.shape) < 0.03
    tipo[pick] = rng.integers(0, 4, size=int(pick.sum()))
    fi = np.asfortranarray(rng.standard_normal((jx + 2, jy + 2, jz + 2)))
    return dict(x=x, y=y, z=z, tipo=tipo, fi=fi, rhs=S.divergence_rhs(jx, jy, jz, 9))


def test_oracle_potenziale_ibm_rules():
    tipo = np.full((4, 4, 4), 2, dtype=np.int32)
    tipo[1, 1, 1] = 0
    tipo[2, 1, 1] = 1
    tipo[1, 2, 1] = 1
    tipo[2, 2, 2] = 0  # no IB neighbour: keeps its value
    fi = np.arange(64, dtype=np.float64).reshape(4, 4, 4)
    out = potenziale_ibm(tipo, fi)
    assert out[1, 1, 1] == (fi[2, 1, 1] + fi[1, 2, 1]) / 2
    assert out[2, 2, 2] == fi[2, 2, 2]
    changed = np.argwhere(out != fi)
    assert changed.tolist() == [[1, 1, 1]]


@pytest.mark.gpu
def test_device_potenziale_ibm_bit_exact(case):
    from ples_gb300 import mg
    with mg.Multigrid(case["x"], case["y"], case["z"], tipo=case["tipo"]) as m:
        got = m.potenziale_ibm(case["fi"])
    want = potenziale_ibm(case["tipo"], case["fi"])
    assert np.array_equal(got, want)
    assert not np.array_equal(got, case["fi"])


@pytest.mark.gpu
def test_stop_test_over_fluid_cells(case):
    from ples_gb300 import mg
    x, y, z = case["x"], case["y"], case["z"]
    with mg.Multigrid(x, y, z) as m:
        f0, s0 = m.solve(case["rhs"], rel_tol=1e-10)
    with mg.Multigrid(x, y, z, tipo=case["tipo"]) as m:
        f1, s1 = m.solve(case["rhs"], rel_tol=1e-10)
        with mg.Batch([m]) as b:  # the batched solve takes the same stop test
            fb, sb = b.solve([case["rhs"]], rel_tol=1e-10)
    assert np.abs(fb[0] - f1).max() <= 1e-9 * np.abs(f1).max()
    assert sb[0]["max_residual"] == pytest.approx(s1["max_residual"], rel=1e-2)
    assert np.array_equal(f0, f1) and s0["rel_residual"] == s1["rel_residual"]
    assert s1["max_residual"] <= s0["max_residual"]
    r, _ = Oracle(x, y, z, islor=1).true_residual(f1, case["rhs"] - case["rhs"].mean())
    assert s1["max_residual"] == pytest.approx(masked_max(case["tipo"], r), rel=1e-2)


@pytest.mark.gpu
def test_potenziale_ibm_needs_tipo(case):
    from ples_gb300 import mg
    with mg.Multigrid(case["x"], case["y"], case["z"]) as m:
        with pytest.raises(mg.PlesMGError):
            m.potenziale_ibm(case["fi"])
