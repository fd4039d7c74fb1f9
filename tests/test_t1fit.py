"""T1 fit (fit.py restatement) against the reference example's own fit outputs.

t1_gaas_example.npz holds the S_z(t) of the reference's GaAs example run and the sfit.out /
tau_t.dat that the reference's fit.py produced from it (tests/golden/make_t1_golden.py). The fitted
curve agrees to the fit's convergence tolerance (scipy leastsq xtol 1.49e-8 on beta); the two-point
lifetimes are closed-form and agree to rounding. The converged lifetime (tau_conv) is the optimum of
the same least-squares problem to machine precision: its gradient vanishes to rounding and a
tightly converged general solver lands on it.
"""
import os

import numpy as np

from conftest import GOLDEN
from denmat_dynm_development_gb300.t1fit import AU_TO_PS, fit_t1, write_sfit, write_tau_t


def _golden():
    return np.load(os.path.join(GOLDEN, "t1_gaas_example.npz"))


def test_fit_matches_reference_sfit_and_tau_t(tmp_path):
    g = _golden()
    sz, sfit, tau_t = g["sz"], g["sfit"], g["tau_t"]
    # the reference fitted the first 3.2 ps of the trajectory
    r = fit_t1(sz[:, 0], sz[:, 1], tend=3.25)
    assert r.t_ps.size == sfit.shape[0]
    np.testing.assert_array_equal(r.s, sfit[:, 1])
    assert np.abs(r.t_ps - sfit[:, 0]).max() < 1e-15
    assert np.abs(r.s_fit - sfit[:, 2]).max() / np.abs(sfit[:, 2]).max() < 1e-8
    assert np.abs(r.tau_t - tau_t[:, 1]).max() / np.abs(tau_t[:, 1]).max() < 1e-10
    assert abs(r.tau_cf - r.tau_lsq) / r.tau_lsq < 1e-7
    write_sfit(str(tmp_path / "sfit.out"), r)
    write_tau_t(str(tmp_path / "tau_t.dat"), r)
    back = np.loadtxt(str(tmp_path / "sfit.out"))
    np.testing.assert_allclose(back, np.transpose([r.t_ps, r.s, r.s_fit]), rtol=1e-15)
    # the converged optimum: within leastsq's tolerance of its answer, a stationary point of the
    # residual, and the root of that stationarity condition found by bracketing (brentq to full
    # precision; scipy's least-squares solvers stop on scale-based tolerances near 1e-8 here)
    assert abs(r.tau_conv - r.tau_lsq) / r.tau_lsq < 1e-7
    import scipy.optimize as so
    t, s = r.t_ps, r.s

    def grad(beta):
        m = s[0] * np.exp(-beta * t)
        return np.sum((s - m) * t * m)
    beta = 1.0 / r.tau_conv
    m = s[0] * np.exp(-beta * t)
    assert abs(grad(beta)) <= 1e-12 * np.sum(np.abs((s - m) * t * m))
    root = so.brentq(grad, 0.5 * beta, 2.0 * beta, xtol=1e-300, rtol=4 * np.finfo(float).eps)
    assert abs(1.0 / root - r.tau_conv) / r.tau_conv < 1e-12


def test_fit_recovers_known_lifetimes():
    t_ps = np.linspace(0.0, 20.0, 201)
    s = -3e-4 * np.exp(-t_ps / 7.5)
    r = fit_t1(t_ps / AU_TO_PS, s)
    assert abs(r.tau_lsq - 7.5) < 1e-6 and abs(r.tau_cf - 7.5) < 1e-6
    assert abs(r.tau_conv - 7.5) / 7.5 < 1e-13
    np.testing.assert_allclose(r.tau_t, 7.5, rtol=1e-9)
    # in-plane field: precession at the Larmor frequency of a g = 1 moment (the reference's omega)
    B = 0.5
    om = B / 2.3505175675871e5 / AU_TO_PS
    s2 = 2e-4 * np.exp(-t_ps / 12.0) * np.cos(om * t_ps)  # S(0) is the amplitude the model fixes
    r2 = fit_t1(t_ps / AU_TO_PS, s2, bfield_tesla=B)
    assert abs(r2.tau_lsq - 12.0) / 12.0 < 1e-6
    assert abs(r2.period_lsq - 2 * np.pi / om) / (2 * np.pi / om) < 1e-6
    assert abs(r2.tau_conv - 12.0) / 12.0 < 1e-13
    assert abs(r2.period_conv - 2 * np.pi / om) / (2 * np.pi / om) < 1e-13
    assert abs(r2.phi_conv) < 1e-12


def test_converged_fit_is_stable_under_last_bit_noise():
    """Two trajectories that differ at 1e-13 (the GPU-vs-oracle level) give lifetimes within 1e-10
    through the converged fit, while the fit.py-faithful leastsq answer moves by ~1e-8 (its xtol)."""
    rng = np.random.default_rng(5)
    t_ps = np.linspace(0.0, 3.0, 61)
    s = 1e-4 * np.exp(-t_ps / 40.0) * (1.0 + 0.01 * np.sin(3.0 * t_ps))  # imperfect model
    a = fit_t1(t_ps / AU_TO_PS, s)
    b = fit_t1(t_ps / AU_TO_PS, s * (1.0 + 1e-13 * rng.standard_normal(s.size)))
    assert abs(b.tau_conv - a.tau_conv) / abs(a.tau_conv) < 1e-10
    B = 1.0
    om = B / 2.3505175675871e5 / AU_TO_PS
    s2 = 1e-4 * np.exp(-t_ps / 40.0) * np.cos(om * t_ps + 0.05) * (1.0 + 0.01 * t_ps)
    a2 = fit_t1(t_ps / AU_TO_PS, s2, bfield_tesla=B)
    b2 = fit_t1(t_ps / AU_TO_PS, s2 * (1.0 + 1e-13 * rng.standard_normal(s2.size)), bfield_tesla=B)
    assert abs(b2.tau_conv - a2.tau_conv) / abs(a2.tau_conv) < 1e-10
    assert abs(b2.period_conv - a2.period_conv) / abs(a2.period_conv) < 1e-10


def test_fit_range_and_errors():
    t_ps = np.linspace(0.0, 10.0, 101)
    s = np.exp(-t_ps / 3.0)
    r = fit_t1(t_ps / AU_TO_PS, s, tstart=2.0, tend=6.0)
    assert r.t_ps[0] == 0.0 and abs(r.t_ps[-1] - 4.0) < 1e-9
    assert abs(r.tau_lsq - 3.0) < 1e-6
    try:
        fit_t1(t_ps / AU_TO_PS, s, tstart=50.0)
    except ValueError:
        pass
    else:
        raise AssertionError("empty fitting range must raise")
