"""The outer stop rule of the mixed-precision defect correction (host
logic, no GPU): stop when the error estimate kappa * ||r|| is below
error_tol * ||F64(u)||, or when the defect alone is below refine_tol."""
import pytest

from pbte_gb300.mixed import MixedOptions, refined


def test_before_any_correction_kappa0_stands_in():
    o = MixedOptions()
    # kappa0 = 100: a restart from a converged state (defect ~5e-13) stops
    assert refined(5e-13, 1.0, None, o)
    assert not refined(2e-11, 1.0, None, o)
    assert not refined(1.0, 1.0, None, o)


def test_error_estimate_scales_with_the_amplification():
    o = MixedOptions()
    # well conditioned (kappa ~ 1): a defect of 1e-9 is enough
    assert refined(0.9e-9, 1.0, 1.0, o)
    # ill conditioned (kappa ~ 1e3): the same defect is not, 1e-12 is
    assert not refined(0.9e-9, 1.0, 1e3, o)
    assert refined(0.9e-12, 1.0, 1e3, o)
    # relative to ||F64(u)||
    assert refined(0.9e-5, 1e4, 1.0, o)


def test_options_tight_comparator_and_unknown_names():
    tight = MixedOptions(refine_tol=1e-13, error_tol=0.0)
    assert not refined(1e-12, 1.0, 1.0, tight) and refined(1e-14, 1.0, 1.0, tight)
    with pytest.raises(TypeError):
        MixedOptions(refine=1e-3)


def test_amplification_of_a_cycle_factor():
    """1 / sigma_min of the triangular factor: with R from the QR of a
    matrix, the norm of that matrix's inverse."""
    import numpy as np

    from pbte_gb300.krylov import amplification
    rng = np.random.default_rng(3)
    A = np.eye(40) + 0.1 * rng.standard_normal((40, 40))
    A[:, 0] *= 1e-3                                  # one slow mode
    R = np.linalg.qr(A)[1]
    assert np.isclose(amplification(R), np.linalg.norm(np.linalg.inv(A), 2), rtol=1e-10)
    assert amplification(np.zeros((0, 0))) == 0.0
