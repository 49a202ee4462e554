"""Device Boys function against the reference's own values and mpmath."""

import cmath

import numpy as np
import pytest

import giaoint_gb300 as gi
from giaoint_gb300.boys import boys_many

pytestmark = pytest.mark.gpu


def test_boys_matches_reference_map_and_reachable_domain(golden):
    cases = golden.boys["cases"]
    z = np.array([complex(*c["z"]) for c in cases])
    vals, region = boys_many(z, 32)
    for k, case in enumerate(cases):
        ref = np.array([complex(*v) for v in case["reference"]])
        err = np.abs(vals[k] - ref)
        assert np.all(err <= 3e-14 + 8e-13 * np.abs(ref)), (case["z"], err.max())
        assert region[k] == case["region"]
        for n, mp in zip(golden.boys["mpmath_orders"], case["mpmath"], strict=True):
            e = complex(*mp)
            assert abs(vals[k][n] - e) <= 3e-14 + 8e-13 * abs(e)


@pytest.mark.parametrize("maximum_order", [0, 3, 12, 32])
def test_boys_orders_individually(golden, maximum_order):
    for case in golden.boys["cases"][:14]:
        v = gi.boys(complex(*case["z"]), maximum_order)
        ref = np.array([complex(*x) for x in case["reference"][: maximum_order + 1]])
        assert np.all(np.abs(v - ref) <= 3e-14 + 8e-13 * np.abs(ref))


def test_scaled_and_domain_errors(golden):
    for case in golden.boys["scaled"]:
        v = gi.boys(complex(*case["z"]), 16, scaled=True)
        ref = np.array([complex(*x) for x in case["reference"]])
        np.testing.assert_allclose(v, ref, atol=2e-14, rtol=8e-13)
    with pytest.raises(gi.BoysNumericalError, match="outside the verified"):
        gi.boys(10.0 + 500.0j, 4)
    with pytest.raises(gi.BoysNumericalError, match="outside the verified"):
        gi.boys(160.001j, 4)
    with pytest.raises(ValueError, match="through 32"):
        gi.boys(1.0, 33)


@pytest.mark.parametrize("argument", [0.2 + 0.4j, 3.0 - 7.0j, -12.0 + 6.0j])
def test_recurrence_residual_and_conjugation(argument):
    values = gi.boys(argument, 20)
    np.testing.assert_allclose(gi.boys(argument.conjugate(), 20), values.conj(), atol=2e-14, rtol=4e-13)
    e = cmath.exp(-argument)
    for n in range(20):
        r = (2 * n + 1) * values[n] - e - 2 * argument * values[n + 1]
        assert abs(r) <= 3e-13 * max(1.0, abs((2 * n + 1) * values[n]) + abs(e))


def test_dense_grid_against_oracle(oracle):
    """Every region of the device method (grid, asymptotic, quadrature) vs the oracle."""
    rng = np.random.default_rng(5)
    z = np.concatenate([
        rng.uniform(-16, 108, 400) + 1j * rng.uniform(-12, 12, 400),
        rng.uniform(-2, 2, 100) + 1j * rng.uniform(-2, 2, 100),
        rng.uniform(100, 400, 50) + 1j * rng.uniform(-20, 20, 50),
        rng.uniform(-100, 100, 30) + 1j * rng.uniform(-40, 40, 30),
    ])
    z = z[np.abs(z) <= 150]
    for nmax in (0, 4, 8, 16):
        vals, _ = boys_many(z, nmax)
        for k in range(len(z)):
            ref, _ = oracle.boys(complex(z[k]), nmax)
            # both sides are quadratures off the grid (reference tolerance 7.5e-14
            # per step): allow 2e-12 relative there, the reference tests' bar elsewhere
            off_grid = not (-16 <= z[k].real <= 108 and abs(z[k].imag) <= 12)
            rtol = 2e-12 if off_grid else 8e-13
            assert np.all(np.abs(vals[k] - ref) <= 3e-14 + rtol * np.abs(ref)), (z[k], nmax)
