"""The outer residual of mixed-precision solves in double-float arithmetic
(products and sums of float pairs on the FP32 pipe, FP64 only for the
differences of x), through the C ABI.

Tolerances: on random fields, where the residual is as large as its terms,
the double-float residual agrees with the FP64 kernel's within 1e-12 of the
largest |r| (the products carry about 2^-47 of their size, 7e-15, against
2^-53 in FP64).  On a smooth field near a solution, where r is small against
its terms, it agrees within 1e-12 of the terms' size: L(|x|) bounds it.  The
scaling by powers of two makes whole solves invariant to the units: a
right-hand side times 2^40 or 2^-40 gives the same solution times the same
power, bit for bit, in the same outer iterations.
"""
import numpy as np
import pytest

from ples_gb300 import mg
from ples_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def _fields(dims, seed, smooth):
    rng = np.random.default_rng(seed)
    jx, jy, jz = dims
    if smooth:
        i = np.arange(jx + 2)[:, None, None]
        j = np.arange(jy + 2)[None, :, None]
        k = np.arange(jz + 2)[None, None, :]
        pr = 1e4 + 50.0 * np.sin(2 * np.pi * i / jx) * np.cos(np.pi * j / jy) + 3.0 * np.cos(2 * np.pi * k / jz)
        pr = pr + 1e-6 * rng.standard_normal((jx + 2, jy + 2, jz + 2))
    else:
        pr = rng.standard_normal((jx + 2, jy + 2, jz + 2))
    rh = rng.standard_normal((jx, jy, jz))
    return np.asfortranarray(pr), np.asfortranarray(rh)


@pytest.mark.parametrize("smooth", [False, True])
@pytest.mark.parametrize("walls", [False, True])
def test_double_float_outer_residual_matches_fp64(smooth, walls):
    dims = (64, 32, 48)
    x, y, z = S.wavy_channel_grid(*dims, 0.1, 2.5)
    pr, rh = _fields(dims, 7, smooth)
    kw = dict(ip=1, kp=0) if walls else {}
    with mg.Multigrid(x, y, z, **kw) as m:
        r64 = m.residual(1, pr, rh, "fp64")
        rdf = m.residual(1, pr, rh, "outer")
        # the terms' size: the operator applied to |pr|, plus |rh|
        scale = np.abs(m.residual(1, np.abs(pr), np.zeros_like(rh), "fp64")).max() + np.abs(rh).max()
    err = np.abs(rdf - r64).max()
    if smooth:
        assert err <= 1e-12 * scale, (err, scale)
    else:
        assert err <= 1e-12 * np.abs(r64).max(), (err, np.abs(r64).max())


def test_fp64_handle_outer_residual_is_the_fp64_kernel():
    dims = (32, 16, 32)
    x, y, z = S.wavy_channel_grid(*dims, 0.05, 2.0)
    pr, rh = _fields(dims, 8, False)
    with mg.Multigrid(x, y, z, precision="fp64") as m:
        a = m.residual(1, pr, rh, "fp64")
        b = m.residual(1, pr, rh, "outer")
        with pytest.raises(mg.PlesMGError):
            m.residual(2, pr[:18, :10, :18], rh[:16, :8, :16], "outer")
    np.testing.assert_allclose(b, a, rtol=0, atol=1e-13 * np.abs(a).max())


@pytest.mark.parametrize("e", [40, -40])
def test_solve_is_invariant_to_power_of_two_units(e):
    dims = (64, 32, 64)
    x, y, z = S.wavy_channel_grid(*dims, 0.08, 2.2)
    rhs = S.divergence_rhs(*dims, seed=9)
    with mg.Multigrid(x, y, z) as m:
        f0, s0 = m.solve(rhs, rel_tol=1e-10)
        f1, s1 = m.solve(np.ldexp(rhs, e), rel_tol=1e-10)
    assert s0["status"] == mg.OK and s1["status"] == mg.OK
    assert s1["outer_iterations"] == s0["outer_iterations"]
    np.testing.assert_array_equal(f1, np.ldexp(f0, e))
