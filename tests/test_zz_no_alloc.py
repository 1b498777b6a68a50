"""ples_mg_residual_norms_device, the entry point that allocates no device
memory, against ples_mg_apply_residual (level 1, FP64) on the same inputs.

Named to be collected last, so that it also runs after every other GPU test
in the same process; it passes alone in a fresh process as well.  Two calls
in a row with different inputs show that the shared scratch carries nothing
from one call to the next.  Cases: a periodic channel on an FP64 and on a
mixed-precision handle, x walls (ghosts filled by ples_mg_apply_ghost_fill
first), an immersed-boundary mask (solid cells are removed rows: r = 0
there) and PLES cell types (the max runs over the fluid cells, tipo >= 2,
as the stop test of multi with bodyforce = 1).
"""
import numpy as np
import pytest

from oracle.ibm import masked_max
from ples_gb300 import mg, synthetic

pytestmark = pytest.mark.gpu

# FP64 with a different summation order than the reference kernel
TOL = 1e-12
DIMS = (64, 32, 64)


def _tipo(rng):
    jx, jy, jz = DIMS
    t = np.full((jx + 2, jy + 2, jz + 2), 2, dtype=np.int32, order="F")
    t[10:20, 5:12, 20:30] = 0
    t[9, 5:12, 20:30] = 1
    pick = rng.random(t.shape) < 0.05
    t[pick] = rng.integers(0, 4, size=int(pick.sum()))
    t[12, 7, 25] = 0  # the cell that gets the planted residual
    return t


CASES = {
    "fp64": dict(precision="fp64"),
    "mixed": dict(precision="mixed"),
    "x_walls": dict(precision="fp64", ip=1),
    "mask": dict(precision="mixed", solid=True),
    "tipo": dict(precision="mixed", tipo=True),
}


@pytest.mark.parametrize("case", list(CASES))
def test_residual_norms_without_allocation_match_apply_residual(case):
    torch = pytest.importorskip("torch")
    jx, jy, jz = DIMS
    opts = dict(CASES[case])
    x, y, z = synthetic.wavy_channel_grid(jx, jy, jz, 0.05, 2.0)
    rng = np.random.default_rng(11)
    solid = tipo = None
    if opts.pop("solid", False):
        solid = synthetic.sphere_mask(x, y, z, n=4, rmin=0.3, rmax=0.5, seed=5)
        opts["solid"] = solid
    if opts.pop("tipo", False):
        tipo = _tipo(rng)
        opts["tipo"] = tipo
    walls = opts.get("ip", 0) == 1
    with mg.Multigrid(x, y, z, **opts) as m:
        for call in range(2):
            fi = np.asfortranarray(rng.standard_normal((jx + 2, jy + 2, jz + 2)) * (1.0 + call))
            if walls:  # the ghost layer the caller hands in: the wall relations' fixed point
                fi = m.ghost_fill(1, fi)
            rhs = np.asfortranarray(rng.standard_normal((jx, jy, jz)))
            if tipo is not None:  # the largest |r| on a solid cell, which the stop test skips
                rhs[11, 6, 24] += 1e3
            r_ref = m.residual(1, fi, rhs, "fp64")
            if solid is not None:
                r_ref[solid] = 0.0
            d_fi = torch.from_numpy(fi.ravel(order="F").copy()).to("cuda:0")
            d_rhs = torch.from_numpy(rhs.ravel(order="F").copy()).to("cuda:0")
            d_r = torch.full((jx * jy * jz,), float("nan"), dtype=torch.float64, device="cuda:0")
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info(0)[0]
            launches0 = m.counters()["launches"]
            ss, mx = m.residual_norms_device(d_fi.data_ptr(), d_rhs.data_ptr(), d_r.data_ptr())
            free1 = torch.cuda.mem_get_info(0)[0]
            assert m.counters()["launches"] == launches0 + 2
            assert free1 == free0, "device memory changed during the call"
            r = d_r.cpu().numpy().reshape((jx, jy, jz), order="F")
            scale = float(np.abs(r_ref).max())
            assert np.abs(r - r_ref).max() <= TOL * scale
            if solid is not None:
                assert np.all(r[solid] == 0.0)
            ss_ref = float((r_ref ** 2).sum())
            assert abs(ss - ss_ref) <= TOL * ss_ref
            mx_ref = masked_max(tipo, r_ref) if tipo is not None else scale
            assert abs(mx - mx_ref) <= TOL * mx_ref
            if tipo is not None:
                assert mx_ref < 0.5 * scale  # the fluid-only max is not the max over all cells
            # without the r output the norms are the same
            ss2, mx2 = m.residual_norms_device(d_fi.data_ptr(), d_rhs.data_ptr())
            assert ss2 == ss and mx2 == mx
