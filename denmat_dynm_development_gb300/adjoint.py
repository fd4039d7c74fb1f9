"""Gradients of the spin trajectory with respect to per-mode coupling scales (reverse mode on the GPU).

The pair operators are taken as a linear combination of fixed operator sets,

    P1 = sum_m theta_m P1^(m),   P2 = sum_m theta_m P2^(m),

one set per phonon mode (a scale of the mode's |g|^2) and one for the impurity term (theta = n_imp
scale, the |n_i V_cell| that DMD folds into P, ElectronImpurity.cpp:38-39). The observed totals
S(t_i) of an observable (S_z: observable.h:301-366) after RK4 steps are a function of theta;
``ModeScaledRK4.gradient`` returns dJ/dtheta for J = sum_i w_i S(t_i) from one call of the
library's adjoint (``dmd_adjoint_rk4``: the discrete adjoint of RK4 with the transposed k-pair
contraction, checkpoints every ``checkpoint`` steps), and ``sz_trajectory`` wraps it as a
``torch.autograd.Function`` so that any differentiable function of the trajectory (a fitted T1,
``t1_loglinear``) can be back-propagated to theta.

dJ/dtheta_m = Re sum conj(dJ/dP) P^(m) over both operators and all pairs, where dJ/dP is the
library's gradient with respect to the folded operators.
"""
from __future__ import annotations

import numpy as np

from .dmd import LindbladGPU


class ModeScaledRK4:
    """S(t_i) of a system whose pair operators are sum_m theta_m P^(m), as a function of theta.

    P1_modes, P2_modes: complex128 [nmodes][nkpair][nb^4] in DMD's layout. obs: the observable
    [nk][nb_dm^2] (S_z: the spin matrices' z component), f_obs: occupations subtracted on its
    diagonal, ob_prefac: 1 / (nk_full cell_size_cmd); S is summed over bands [obs_bstart, bend).
    obs_steps: ascending step counts at which S is observed (0 = the initial state)."""

    def __init__(self, *, nk, nb_dm, bstart, bend, e_dm, k1st, k2nd, P1_modes, P2_modes, prefac_eph, y0, dt,
                 nsteps, obs_steps, obs, f_obs, ob_prefac, obs_bstart=0, t0=0.0, Hcoh=None, picture="interaction",
                 expt=1, precision="f64x", checkpoint=200, device=0):
        self.sys = dict(nk=nk, nb_dm=nb_dm, bstart=bstart, bend=bend, e_dm=e_dm, k1st=k1st, k2nd=k2nd,
                        prefac_eph=prefac_eph, Hcoh=Hcoh, picture=picture, expt=expt, precision=precision,
                        device=device)
        self.P1m = np.asarray(P1_modes, np.complex128)
        self.P2m = np.asarray(P2_modes, np.complex128)
        if self.P1m.shape != self.P2m.shape or self.P1m.ndim != 3:
            raise ValueError("P1_modes and P2_modes must both be [nmodes][nkpair][nb^4]")
        self.nmodes = self.P1m.shape[0]
        self.y0 = np.ascontiguousarray(y0, np.float64)
        self.t0, self.dt, self.nsteps = float(t0), float(dt), int(nsteps)
        self.obs_steps = np.asarray(obs_steps, np.int64)
        if self.obs_steps.size and (np.any(np.diff(self.obs_steps) < 0) or self.obs_steps[0] < 0
                                    or self.obs_steps[-1] > self.nsteps):
            raise ValueError("obs_steps must be ascending in [0, nsteps]")
        self.obs, self.f_obs, self.ob_prefac = obs, f_obs, float(ob_prefac)
        self.obs_bstart = int(obs_bstart)
        self.checkpoint = int(checkpoint)

    def operators(self, theta):
        th = np.asarray(theta, np.float64)
        if th.shape != (self.nmodes,):
            raise ValueError("theta must have %d entries" % self.nmodes)
        return np.tensordot(th, self.P1m, 1), np.tensordot(th, self.P2m, 1)

    def _handle(self, theta, adjoint):
        P1, P2 = self.operators(theta)
        g = LindbladGPU(P1=P1.reshape(-1), P2=P2.reshape(-1), adjoint=adjoint, **self.sys)
        g.set_observable(0, self.obs, self.f_obs, self.ob_prefac)
        return g

    def forward(self, theta):
        """S at the observed steps (the library's RK4 stepper)."""
        with self._handle(theta, False) as g:
            g.set_state(self.t0, self.y0)
            out, cur = [], 0
            for s in self.obs_steps:
                if s > cur:
                    g.rk4(self.dt, int(s - cur))
                    cur = int(s)
                out.append(g.measure(0, self.obs_bstart)[0])
        return np.array(out)

    def gradient(self, theta, weights):
        """(S at the observed steps, dJ/dtheta) for J = sum_i weights[i] S(t_i)."""
        w = np.asarray(weights, np.float64)
        with self._handle(theta, True) as g:
            s, dP, _ = g.adjoint_rk4(self.t0, self.y0, self.dt, self.nsteps, self.obs_steps, w, slot=0,
                                     bstart=self.obs_bstart, checkpoint=self.checkpoint)
        grad = np.array([np.vdot(dP[0], self.P1m[m]).real + np.vdot(dP[1], self.P2m[m]).real
                         for m in range(self.nmodes)])
        return s, grad


class StreamedModeScaledRK4:
    """ModeScaledRK4 for systems whose operator sets do not fit in memory together (the 4.19M-pair
    nb = 4 MoS2-like system: 34 GB per set in complex128). The sets come from a source with
    scaled(theta), mode(m) and contract(G) -- ldbd_synth.ModeSets regenerates them chunk by chunk --
    and one device handle (DMD_FLAG_ADJOINT) at theta serves both the gradient and the central
    differences: dmd_add_operators shifts one set's scale in place (P += delta P^(m)), so at most one
    set besides P is on the host at a time and P itself lives only on the device after set-up.

    The gradient is dJ/dtheta_m = Re sum conj(dJ/dP) P^(m): dJ/dP (one more set's worth of memory)
    is written by the library's adjoint into shared memory and contracted by the source's workers."""

    def __init__(self, *, modes, nk, nb_dm, bstart, bend, e_dm, k1st, k2nd, prefac_eph, y0, dt, nsteps, obs_steps,
                 obs, f_obs, ob_prefac, theta, obs_bstart=0, t0=0.0, Hcoh=None, picture="interaction", expt=1,
                 precision="f64x", checkpoint=200, device=0):
        self.modes = modes
        self.nparams = modes.nparams
        self.theta = np.asarray(theta, np.float64)
        if self.theta.shape != (self.nparams,):
            raise ValueError("theta must have %d entries" % self.nparams)
        self.y0 = np.ascontiguousarray(y0, np.float64)
        self.t0, self.dt, self.nsteps = float(t0), float(dt), int(nsteps)
        self.obs_steps = np.asarray(obs_steps, np.int64)
        self.obs_bstart = int(obs_bstart)
        self.checkpoint = int(checkpoint)
        P = modes.scaled(self.theta)
        try:
            self.g = LindbladGPU(nk=nk, nb_dm=nb_dm, bstart=bstart, bend=bend, e_dm=e_dm, k1st=k1st, k2nd=k2nd,
                                 P1=P.a[0], P2=P.a[1], prefac_eph=prefac_eph, Hcoh=Hcoh, picture=picture, expt=expt,
                                 precision=precision, device=device, adjoint=True)
        finally:
            P.close()
        self.g.set_observable(0, obs, f_obs, ob_prefac)

    def close(self):
        if self.g is not None:
            self.g.close()
            self.g = None

    def forward(self):
        """S at the observed steps with the handle's current operators"""
        g = self.g
        g.set_state(self.t0, self.y0)
        out, cur = [], 0
        for s in self.obs_steps:
            if s > cur:
                g.rk4(self.dt, int(s - cur))
                cur = int(s)
            out.append(g.measure(0, self.obs_bstart)[0])
        return np.array(out)

    def gradient(self, weights):
        """(S at the observed steps, dJ/dtheta) at self.theta for J = sum_i weights[i] S(t_i)"""
        import time
        from .ldbd_synth import SharedPair
        w = np.asarray(weights, np.float64)
        G = SharedPair(self.g.npair, self.g.nb4)
        try:
            t0 = time.perf_counter()
            s, _, _ = self.g.adjoint_rk4(self.t0, self.y0, self.dt, self.nsteps, self.obs_steps, w, slot=0,
                                         bstart=self.obs_bstart, checkpoint=self.checkpoint, dP_out=G.a)
            t1 = time.perf_counter()
            grad = self.modes.contract(G)
            self.last_timing = {"adjoint_rk4_s": t1 - t0, "mode_contraction_s": time.perf_counter() - t1}
        finally:
            G.close()
        return s, grad

    def central_differences(self, weights, rel_step=1e-4):
        """dJ/dtheta_m by central differences, h = rel_step * theta_m, each set shifted in place"""
        w = np.asarray(weights, np.float64)
        out = np.zeros(self.nparams)
        for m in range(self.nparams):
            h = rel_step * self.theta[m]
            Pm = self.modes.mode(m)
            try:
                self.g.add_operators(Pm.a[0], Pm.a[1], h)
                jp = float(w @ self.forward())
                self.g.add_operators(Pm.a[0], Pm.a[1], -2.0 * h)
                jm = float(w @ self.forward())
                self.g.add_operators(Pm.a[0], Pm.a[1], h)
            finally:
                Pm.close()
            out[m] = (jp - jm) / (2.0 * h)
        return out


def sz_trajectory(theta, model: ModeScaledRK4):
    """torch: S(t_i) as a differentiable function of theta (a float64 tensor of nmodes entries)."""
    return _SzFn.apply(theta, model)


def _make_fn():
    import torch

    class SzFn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta, model):
            ctx.model = model
            ctx.save_for_backward(theta)
            return torch.as_tensor(model.forward(theta.detach().cpu().numpy()), dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad_s):
            (theta,) = ctx.saved_tensors
            _, g = ctx.model.gradient(theta.detach().cpu().numpy(), grad_s.detach().cpu().numpy())
            return torch.as_tensor(g, dtype=theta.dtype, device=theta.device), None

    return SzFn


class _Lazy:
    fn = None

    def apply(self, *args):
        if _Lazy.fn is None:
            _Lazy.fn = _make_fn()
        return _Lazy.fn.apply(*args)


_SzFn = _Lazy()


def t1_loglinear(t, s):
    """torch: lifetime from the least-squares slope of log|S| against t (t in any unit; T1 in it).
    For S = S0 exp(-t / T1) it is exactly T1."""
    import torch
    y = torch.log(torch.abs(s))
    x = torch.as_tensor(t, dtype=s.dtype, device=s.device)
    xm, ym = x.mean(), y.mean()
    slope = ((x - xm) * (y - ym)).sum() / ((x - xm) ** 2).sum()
    return -1.0 / slope
