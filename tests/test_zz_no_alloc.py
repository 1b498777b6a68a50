"""ples_mg_residual_norms_device, the entry point that allocates no device
memory, against ples_mg_apply_residual (level 1, FP64) on the same inputs.

Named to be collected last, so that it also runs after every other GPU test
in the same process; it passes alone in a fresh process as well.  Two calls
in a row with different inputs show that the shared scratch carries nothing
from one call to the next.
"""
import numpy as np
import pytest

from ples_gb300 import mg, synthetic

pytestmark = pytest.mark.gpu

# FP64 with a different summation order than the reference kernel
TOL = 1e-12


def test_residual_norms_without_allocation_match_apply_residual():
    torch = pytest.importorskip("torch")
    jx, jy, jz = 64, 32, 64
    x, y, z = synthetic.wavy_channel_grid(jx, jy, jz, 0.05, 2.0)
    rng = np.random.default_rng(11)
    with mg.Multigrid(x, y, z, precision="fp64") as m:
        for call in range(2):
            fi = np.asfortranarray(rng.standard_normal((jx + 2, jy + 2, jz + 2)) * (1.0 + call))
            rhs = np.asfortranarray(rng.standard_normal((jx, jy, jz)))
            r_ref = m.residual(1, fi, rhs, "fp64")
            d_fi = torch.from_numpy(fi.ravel(order="F").copy()).to("cuda:0")
            d_rhs = torch.from_numpy(rhs.ravel(order="F").copy()).to("cuda:0")
            d_r = torch.full((jx * jy * jz,), float("nan"), dtype=torch.float64, device="cuda:0")
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info(0)[0]
            launches0 = m.counters()["launches"]
            ss, mx = m.residual_norms_device(d_fi.data_ptr(), d_rhs.data_ptr(), d_r.data_ptr())
            free1 = torch.cuda.mem_get_info(0)[0]
            assert m.counters()["launches"] == launches0 + 2
            if call == 1:  # the first call may load the module on this device
                assert free1 == free0, "device memory changed during the call"
            r = d_r.cpu().numpy().reshape((jx, jy, jz), order="F")
            scale = float(np.abs(r_ref).max())
            assert np.abs(r - r_ref).max() <= TOL * scale
            ss_ref = float((r_ref ** 2).sum())
            assert abs(ss - ss_ref) <= TOL * ss_ref
            assert abs(mx - scale) <= TOL * scale
            # without the r output the norms are the same
            ss2, mx2 = m.residual_norms_device(d_fi.data_ptr(), d_rhs.data_ptr())
            assert ss2 == ss and mx2 == mx
