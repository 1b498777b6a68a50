"""Failure detection of a bounded device wait, without a GPU fault.

The waits on the device are the mbarrier waits of the TMA-staged line
smoother (smoother 2) and the plane waits of the merged-parity 64-line
smoother (form 4096).  ples_mg_set_wait_limit(0) makes each of them give
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


def test_merged_sweep_wait_that_runs_out_and_recovery():
    """The 64-line-tile smoother with both k parities in one launch (form
    4096): an even-k tile waits for the odd planes either side of it.  With
    a wait limit of 0 an even-k tile gives up at its first poll that finds
    them incomplete (of the hundreds of such tiles a solve starts alongside
    the odd-plane tiles, some do), skips its lines and the solve returns
    PLES_MG_DEVICE_TIMEOUT; with the default limit restored the handle solves
    again and gives the field it gave before, bit for bit (the counters of
    the launch are zeroed by its last CTA, also after a timeout)."""
    dims = (128, 64, 128)
    x, y, z = S.wavy_channel_grid(*dims, 0.05, 2.0)
    rhs = S.divergence_rhs(*dims, seed=32)
    with mg.Multigrid(x, y, z) as m:
        m.set_line_threads(1, 4096)
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
