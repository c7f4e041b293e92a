"""Accuracy of the device FP64 helpers (table-driven exponential, Newton
reciprocal) against CUDA's exp and IEEE division on the same GPU. The KMC
rates, barriers and clock use them; the error bars here (a few ulp) sit far
inside the barrier/time tolerances of the parity tests (1e-9 relative)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EXP_MAX_ULP = 4.0
RCP_MAX_ULP = 2.0


@pytest.fixture(scope="module")
def ctx(native):
    from latticemontecarlo_gb300 import api, synthetic as S
    el = ("Al", "Mg", "Zn")
    m = api.Model.from_coefficients(S.make_coefficients(el, 3, calibrate=False), list(el))
    return api.Context(m)


def _run(ctx, fn, x):
    from latticemontecarlo_gb300 import _native as N
    x = np.ascontiguousarray(x, dtype=np.float64)
    fast, ref = np.zeros_like(x), np.zeros_like(x)
    N.check(N.lib.lmc_fastmath_check(ctx._h, fn, N.ptr(x, C.c_double), x.size, N.ptr(fast, C.c_double),
                                     N.ptr(ref, C.c_double)))
    return fast, ref


def _ulp(a, b):
    return np.abs(a - b) / np.spacing(np.abs(b))


def test_exp_accuracy(ctx):
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.uniform(-700, 700, 400_000), rng.uniform(-60, 0, 400_000),  # rate arguments
                        rng.uniform(-1e-3, 1e-3, 50_000), [0.0, -0.0, 1e-300, -1e-300, 699.999, -699.999],
                        np.arange(-2000, 2001) * np.log(2) / 256])  # table nodes
    fast, ref = _run(ctx, 0, x)
    assert np.all(np.isfinite(fast))
    err = _ulp(fast, ref)
    assert err.max() <= EXP_MAX_ULP, (err.max(), x[np.argmax(err)])
    # outside the table range the library exp is used unchanged
    y = np.array([700.0, -700.0, 709.7, -745.0, -800.0, np.inf, -np.inf])
    f2, r2 = _run(ctx, 0, y)
    assert np.array_equal(f2, r2)


def test_reciprocal_accuracy(ctx):
    rng = np.random.default_rng(2)
    mag = 10.0 ** rng.uniform(-30, 30, 500_000)
    x = np.concatenate([mag, -mag, [1.0, 3.0, 64.0, 1e13, 1.2e14, 7.0e-20]])
    fast, ref = _run(ctx, 1, x)
    err = _ulp(fast, ref)
    assert err.max() <= RCP_MAX_ULP, (err.max(), x[np.argmax(err)])
    # outside the FP32 exponent range: IEEE division
    y = np.array([1e-300, 1e300, -1e-300, 0.0, np.inf])
    with np.errstate(divide="ignore"):
        f2, r2 = _run(ctx, 1, y)
    assert np.array_equal(f2, r2)
