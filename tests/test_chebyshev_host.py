"""CPU tests of the Chebyshev method's host mathematics in libelhlprop.so
(Bessel sequence, expansion coefficients); no GPU needed."""
import numpy as np
import pytest

from dynemol_gb300 import api, build

H_BAR = 6.58264e-4


@pytest.fixture(scope="module")
def lib():
    build.build()
    return api.load()


@pytest.mark.parametrize("beta", [0.0, 1e-3, 0.7, 8.4, 37.2, 96.8, 250.0])
def test_bessel_matches_scipy(lib, beta):
    special = pytest.importorskip("scipy.special")
    kmax = int(beta) + 60
    J = api.bessel_j(beta, kmax)
    ref = special.jv(np.arange(kmax + 1), beta)
    assert np.abs(J - ref).max() < 1e-13


@pytest.mark.parametrize("dt,emin,emax", [(1e-4, -31.0, 79.0), (5e-4, -41.0, 215.0), (1e-4, -2.0, 3.0)])
def test_coefficients_reconstruct_propagator(lib, dt, emin, emax):
    """sum_k c_k T_k(x) == exp(-i tau (a + b x)) on [-1, 1]."""
    c = api.chebyshev_coefficients(dt, emin, emax, tol=1e-14)
    tau = dt / H_BAR
    a, b = 0.5 * (emax + emin), 0.5 * (emax - emin)
    x = np.cos(np.linspace(0.0, np.pi, 301))
    T = np.polynomial.chebyshev.chebvander(x, len(c) - 1)
    f = T @ c
    assert np.abs(f - np.exp(-1j * tau * (a + b * x))).max() < 1e-12
    assert len(c) - 1 >= tau * b  # order at least beta


def test_coefficient_arguments(lib):
    with pytest.raises(api.ElhlError):
        api.chebyshev_coefficients(1e-4, 1.0, 1.0)
    with pytest.raises(api.ElhlError):
        api.chebyshev_coefficients(-1e-4, -1.0, 1.0)
