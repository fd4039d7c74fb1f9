"""Spin lifetime T1 from an S(t) trajectory.

Restates the reference's post-processing fit (Examples/RealTime_Example_GaAs_20230105/ld-dmd/t300/
mult8_gauss0.005/dBz/eph-ei/n2e16_ni2e16/fit.py:7-78):

* time column in atomic units converted to ps (x 2.4188843265857e-5, fit.py:13), points kept in
  [tstart, tend] (fit.py:14-15) and shifted to start at 0 (fit.py:17);
* global fit of S(t) = S(0) exp(-beta t) with S(0) fixed to the first sample (fit.py:27-29), done two
  ways like the reference: curve_fit from its default start (beta = 1) and leastsq from beta = 1/100 ps
  (fit.py:21, 39-41); tau = 1/beta; with an in-plane field B the model gains cos(omega t + phi)
  (fit.py:30-32, 42-44) with omega from B (fit.py:23-24);
* the fitted curve from the leastsq parameters (fit.py:53-57);
* time-resolved lifetimes from two-point linear fits of log|S| (fit.py:60-67): tau_i = -1/slope.

Both fits stop at scipy's default tolerances (xtol ~1.5e-8 on beta), so tau_cf and tau_lsq carry
that much convergence noise. tau_conv (and period_conv, phi_conv) is the same least-squares problem
solved to machine precision: Gauss-Newton steps from the leastsq parameters until a step no longer
shrinks the parameters' change below a few ulps. Comparing two trajectories' lifetimes at the 1e-10
level needs tau_conv; tau_cf / tau_lsq stay what the reference's fit.py reports.

The trajectories come from the GPU steppers (S_z sampled by dmd_measure); the function is pure
numpy/scipy and runs on the host.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

AU_TO_PS = 2.4188843265857e-5
TESLA_TO_AU = 1.0 / 2.3505175675871e5


@dataclass
class T1Fit:
    t_ps: np.ndarray          # fitted times, shifted to start at 0 (ps)
    s: np.ndarray             # S(t) on those times
    tau_cf: float             # lifetime from curve_fit (ps)
    tau_lsq: float            # lifetime from leastsq (ps)
    s_fit: np.ndarray         # model evaluated with the leastsq parameters
    tau_t: np.ndarray         # time-resolved lifetimes, len(t_ps) - 1 (ps)
    period_cf: float = float("nan")   # precession period and phase (only with a field)
    period_lsq: float = float("nan")
    phi_cf: float = float("nan")
    phi_lsq: float = float("nan")
    tau_conv: float = float("nan")    # lifetime of the least-squares optimum to machine precision (ps)
    period_conv: float = float("nan")
    phi_conv: float = float("nan")
    conv_iters: int = 0


def load_s(path: str):
    """Columns 0 (time, a.u.) and 1 (S) of an s?_elec_tot.out file (header lines start with '#')."""
    a = np.loadtxt(path, usecols=(0, 1))
    return a[:, 0], a[:, 1]


def fit_t1(t_au, s, tstart: float = 0.0, tend: float = np.inf, bfield_tesla: float = 0.0) -> T1Fit:
    import scipy.optimize as so

    t = np.asarray(t_au, dtype=np.float64) * AU_TO_PS
    keep = (t >= tstart) & (t <= tend)
    t = t[keep]
    if t.size < 2:
        raise ValueError("fit_t1: fewer than two samples in the fitting range")
    t = t - t[0]
    sv = np.asarray(s, dtype=np.float64)[keep]
    s0 = sv[0]
    omega = bfield_tesla * TESLA_TO_AU / AU_TO_PS

    def decay(tt, beta):
        return s0 * np.exp(-beta * tt)

    def decay_cos(tt, beta, om, phi):
        return s0 * np.exp(-beta * tt) * np.cos(om * tt + phi)

    if omega == 0.0:
        p_cf, _ = so.curve_fit(decay, t, sv)
        p_lsq, _ = so.leastsq(lambda p: sv - decay(t, *p), [1.0 / 100.0])
        s_fit = decay(t, p_lsq[0])
        res = T1Fit(t, sv, 1.0 / p_cf[0], 1.0 / p_lsq[0], s_fit, _tau_t(t, sv))
        pc, it = _gauss_newton(lambda p: _decay_jac(t, s0, p), np.array([p_lsq[0]], dtype=np.float64), sv)
        res.tau_conv, res.conv_iters = 1.0 / pc[0], it
    else:
        p_cf, _ = so.curve_fit(decay_cos, t, sv)
        p_lsq, _ = so.leastsq(lambda p: sv - decay_cos(t, *p), [1.0 / 100.0, omega, 0.0])
        s_fit = decay_cos(t, *p_lsq)
        res = T1Fit(t, sv, 1.0 / p_cf[0], 1.0 / p_lsq[0], s_fit, _tau_t(t, sv),
                    period_cf=2 * np.pi / p_cf[1], period_lsq=2 * np.pi / p_lsq[1], phi_cf=p_cf[2], phi_lsq=p_lsq[2])
        pc, it = _gauss_newton(lambda p: _decay_cos_jac(t, s0, p), np.array(p_lsq, dtype=np.float64), sv,
                               floor=np.array([0.0, 0.0, 1.0]))
        res.tau_conv, res.period_conv, res.phi_conv, res.conv_iters = 1.0 / pc[0], 2 * np.pi / pc[1], pc[2], it
    return res


def _decay_jac(t, s0, p):
    """model s0 exp(-beta t), its derivative and its second derivative in beta"""
    m = s0 * np.exp(-p[0] * t)
    return m, (-t * m)[:, None], (t * t * m)[:, None, None]


def _decay_cos_jac(t, s0, p):
    """model s0 exp(-beta t) cos(omega t + phi), its derivatives and second derivatives in
    (beta, omega, phi)"""
    beta, om, phi = p
    ex = s0 * np.exp(-beta * t)
    c, sn = np.cos(om * t + phi), np.sin(om * t + phi)
    m = ex * c
    J = np.stack([-t * m, -t * ex * sn, -ex * sn], axis=1)
    H = np.empty((t.size, 3, 3))
    H[:, 0, 0] = t * t * m
    H[:, 0, 1] = H[:, 1, 0] = t * t * ex * sn
    H[:, 0, 2] = H[:, 2, 0] = t * ex * sn
    H[:, 1, 1] = -t * t * m
    H[:, 1, 2] = H[:, 2, 1] = -t * m
    H[:, 2, 2] = -m
    return m, J, H


def _gauss_newton(model_jac, p, s, max_iter: int = 100, floor=None):
    """Least-squares parameters of s ~ model(p) to machine precision, from a start near the optimum.

    Newton steps on the stationarity condition J^T r = 0 (r = s - model) with the exact Hessian
    J^T J - sum_i r_i d2 model_i, which converge quadratically whatever the size of the residual
    (Gauss-Newton alone converges only linearly when the model does not fit the data exactly). A
    large step (above 1e-6 of a parameter) is halved until the sum of squared residuals does not rise,
    so the iteration stays at the local optimum next to the start; closer in, the residual is flat to
    rounding and steps are taken as they come. While the exact Hessian is not positive definite the
    Gauss-Newton matrix J^T J is used. The loop stops once a step is below 4 ulps of every parameter
    (of max(|p|, floor) for a parameter that may be zero, such as a phase), or when a small step no
    longer shrinks (the rounding floor of the gradient): the last iterate is then the optimum up to
    that floor."""
    p = np.array(p, dtype=np.float64)
    floor = np.zeros_like(p) if floor is None else np.asarray(floor, dtype=np.float64)
    scale = lambda q: np.maximum(np.maximum(np.abs(q), floor), 1e-300)  # noqa: E731
    m, J, Hm = model_jac(p)
    r = s - m
    ssr = float(r @ r)
    prev = np.inf
    it = 0
    for it in range(1, max_iter + 1):
        g = J.T @ r
        H = J.T @ J - np.einsum("i,ijk->jk", r, Hm)
        try:
            np.linalg.cholesky(H)
            dp = np.linalg.solve(H, g)
        except np.linalg.LinAlgError:
            dp = np.linalg.lstsq(J, r, rcond=None)[0]
        size = float(np.max(np.abs(dp) / scale(p)))
        lam = 1.0
        while True:
            pn = p + lam * dp
            mn, Jn, Hn = model_jac(pn)
            rn = s - mn
            ssrn = float(rn @ rn)
            if lam * size < 1e-6 or ssrn <= ssr:
                break
            lam *= 0.5
        p, J, Hm, r, ssr = pn, Jn, Hn, rn, ssrn
        size = lam * size
        if size <= 4 * np.finfo(np.float64).eps:
            break
        if size < 1e-10 and size > 0.5 * prev:
            break  # the steps stopped shrinking: at the rounding floor
        prev = size
    return p, it


def _tau_t(t, s):
    ls = np.log(np.abs(s))
    out = np.empty(t.size - 1)
    for i in range(t.size - 1):
        out[i] = -1.0 / np.polyfit(t[i:i + 2], ls[i:i + 2], 1)[0]
    return out


def write_sfit(path: str, r: T1Fit) -> None:
    """The reference's sfit.out: columns t (ps), S, fitted S."""
    np.savetxt(path, np.transpose([r.t_ps, r.s, r.s_fit]))


def write_tau_t(path: str, r: T1Fit) -> None:
    """The reference's tau_t.dat: columns t (ps), time-resolved tau (ps)."""
    np.savetxt(path, np.transpose([r.t_ps[:-1], r.tau_t]))
