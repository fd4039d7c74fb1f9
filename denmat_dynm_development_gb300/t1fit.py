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
    else:
        p_cf, _ = so.curve_fit(decay_cos, t, sv)
        p_lsq, _ = so.leastsq(lambda p: sv - decay_cos(t, *p), [1.0 / 100.0, omega, 0.0])
        s_fit = decay_cos(t, *p_lsq)
        res = T1Fit(t, sv, 1.0 / p_cf[0], 1.0 / p_lsq[0], s_fit, _tau_t(t, sv),
                    period_cf=2 * np.pi / p_cf[1], period_lsq=2 * np.pi / p_lsq[1], phi_cf=p_cf[2], phi_lsq=p_lsq[2])
    return res


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
