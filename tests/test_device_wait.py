"""Failure detection of a bounded device wait, without a GPU fault.

The only waits on the device are the mbarrier waits of the TMA-staged line
smoother (smoother 2).  ples_mg_set_wait_limit(0) makes each of them give
up at its first poll: the CTA records the failure, waits with the default
limits for the copies it still has in flight and leaves; the host reads the
flag and the solve returns PLES_MG_DEVICE_TIMEOUT.  With the default limit
restored, the same handle solves again and gives the field it gave before
the timeout, bit for bit (its work buffers are rebuilt by every solve).
"""
import numpy as np
import pytest

from ples_gb300 import mg
from ples_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def test_wait_that_runs_out_reports_device_timeout_and_the_handle_recovers():
    dims = (64, 32, 64)
    x, y, z = S.wavy_channel_grid(*dims, 0.05, 2.0)
    rhs = S.divergence_rhs(*dims, seed=31)
    with mg.Multigrid(x, y, z, smoother=2) as m:
        f0, s0 = m.solve(rhs, rel_tol=1e-10)
        assert s0["status"] == mg.OK
        m.set_wait_limit(0)
        with pytest.raises(mg.PlesMGError) as e:
            m.solve(rhs, rel_tol=1e-10)
        assert e.value.code == mg.DEVICE_TIMEOUT
        m.set_wait_limit(-1)
        f1, s1 = m.solve(rhs, rel_tol=1e-10)
        assert s1["status"] == mg.OK
    assert np.array_equal(f0, f1)


def test_wait_limit_arguments():
    x, y, z = S.wavy_channel_grid(32, 16, 32, 0.05, 2.0)
    with mg.Multigrid(x, y, z) as m:
        with pytest.raises(mg.PlesMGError):
            m.set_wait_limit(1 << 40)
        m.set_wait_limit(5)
        m.set_wait_limit(-1)
