"""Reverse-mode gradients (dmd_adjoint_rk4) against central finite differences.

The objective is J = sum_i w_i S_z(t_i) over fixed RK4 steps. The adjoint's dJ/dP (the gradient with
respect to the stored pair operators) and dJ/dy0 are checked along random directions against
central differences (h = 1e-4) of the GPU forward; the per-mode gradient dJ/dtheta of a synthetic
system with P = sum_m theta_m P^(m) (6 phonon modes + the impurity term) against central
differences of the GPU forward and of the FP64 oracle; and the torch.autograd wrapper through a
fitted lifetime. Tolerance: 1e-5 relative (the target for the adjoint), cases without the
equilibrium-drift subtraction.
"""
import dataclasses
import os

import numpy as np
import pytest

from conftest import GOLDEN

FD_H = 1e-4
TOL = 1e-5


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as G
    G.build()


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / np.abs(b).max())


def _gpu(s, P1=None, P2=None, adjoint=False, precision="f64"):
    from denmat_dynm_development_gb300.dmd import LindbladGPU
    g = LindbladGPU(nk=s.nk, nb_dm=s.nb_dm, bstart=s.bstart, bend=s.bend, e_dm=s.e_dm, k1st=s.k1st, k2nd=s.k2nd,
                    P1=s.P1 if P1 is None else P1, P2=s.P2 if P2 is None else P2, prefac_eph=s.prefac_eph,
                    Hcoh=s.Hcoh, picture=s.picture_schrodinger, expt=s.expt, precision=precision, adjoint=adjoint)
    g.set_observable(0, s.smat[:, 2, :], s.f_dm, s.ob_prefac)
    return g


def _objective(s, y0, dt, steps, w, P1=None, P2=None):
    with _gpu(s, P1, P2) as g:
        g.set_state(s.t0, y0)
        out, cur = [], 0
        for st in steps:
            if st > cur:
                g.rk4(dt, int(st - cur))
                cur = int(st)
            out.append(g.measure(0, s.nv_dm)[0])
    return float(np.dot(w, out)), np.array(out)


@pytest.mark.gpu
@pytest.mark.parametrize("keep", ["1", "0"])
@pytest.mark.parametrize("case", ["nb2_eimp_B", "nb2_schrod", "nb4_eimp_B", "nb2_window"])
def test_adjoint_directional_derivatives_vs_fd(case, keep, oracle, built, monkeypatch):
    """keep = 1: the forward pass keeps every stage (these sizes fit); keep = 0: the backward pass
    recomputes stretches of 7 steps from checkpoints"""
    monkeypatch.setenv("DMD_ADJ_KEEP_ALL", keep)
    s = oracle.load(os.path.join(GOLDEN, case))
    rng = np.random.default_rng(3)
    dt = 2.0 * oracle.fs
    steps = np.array([0, 9, 20, 33])
    w = rng.standard_normal(steps.size)
    y0 = oracle.y_of(s.dm0)
    with _gpu(s, adjoint=True) as g:
        sv, dP, dy0 = g.adjoint_rk4(s.t0, y0, dt, int(steps[-1]), steps, w, slot=0, bstart=s.nv_dm, checkpoint=7,
                                    want_dy0=True)
    J0, s_fwd = _objective(s, y0, dt, steps, w)
    assert rel(sv, s_fwd) < 1e-12
    # dJ/dP along a random complex direction of both operators
    n = s.P1.size
    d1 = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * np.abs(s.P1).max()
    d2 = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * np.abs(s.P2).max()
    jp, _ = _objective(s, y0, dt, steps, w, s.P1 + FD_H * d1, s.P2 + FD_H * d2)
    jm, _ = _objective(s, y0, dt, steps, w, s.P1 - FD_H * d1, s.P2 - FD_H * d2)
    fd = (jp - jm) / (2 * FD_H)
    ad = np.vdot(dP[0].reshape(-1), d1).real + np.vdot(dP[1].reshape(-1), d2).real
    print("%s dJ/dP: adjoint %.12g fd %.12g rel %.3g" % (case, ad, fd, abs(ad - fd) / abs(fd)))
    assert abs(ad - fd) <= TOL * abs(fd)
    # dJ/dy0 along a random Hermitian direction (the state stays Hermitian)
    dm = rng.standard_normal(s.dm0.shape) + 1j * rng.standard_normal(s.dm0.shape)
    dm = dm.reshape(s.nk, s.nb_dm, s.nb_dm)
    dm = 0.5 * (dm + np.conj(np.swapaxes(dm, 1, 2)))
    dy = oracle.y_of(dm.reshape(s.nk, -1)) * 1e-3
    jp, _ = _objective(s, y0 + FD_H * dy, dt, steps, w)
    jm, _ = _objective(s, y0 - FD_H * dy, dt, steps, w)
    fd = (jp - jm) / (2 * FD_H)
    ad = float(np.dot(dy0, dy))
    print("%s dJ/dy0: adjoint %.12g fd %.12g rel %.3g" % (case, ad, fd, abs(ad - fd) / abs(fd)))
    assert abs(ad - fd) <= TOL * abs(fd)


@pytest.mark.gpu
@pytest.mark.parametrize("nb_dm,bstart,bend,npair,picture", [(3, 0, 3, 90, 0), (1, 0, 1, 60, 1), (3, 1, 2, 50, 1)])
def test_adjoint_generic_windows_vs_fd(nb_dm, bstart, bend, npair, picture, oracle, built):
    """nb = 1 and 3 windows (FP64 handles on the per-thread pair kernels, one window inside the density
    matrix), both pictures, random operators and a random Hermitian observable: dJ/dP and dJ/dy0 of
    the adjoint against central differences of the GPU forward"""
    from test_gpu_parity import _random_system
    s = _random_system(oracle, 17, nb_dm, bstart, bend, npair, seed=100 + nb_dm * 10 + npair, picture=picture)
    rng = np.random.default_rng(11)
    ob = rng.standard_normal((s.nk, nb_dm, nb_dm)) + 1j * rng.standard_normal((s.nk, nb_dm, nb_dm))
    ob = 0.5 * (ob + np.conj(np.swapaxes(ob, 1, 2)))
    smat = np.zeros((s.nk, 3, nb_dm * nb_dm), np.complex128)
    smat[:, 2, :] = ob.reshape(s.nk, -1)
    s = dataclasses.replace(s, smat=smat)
    dt = 2.0 * oracle.fs
    steps = np.array([0, 6, 13, 21])
    w = rng.standard_normal(steps.size)
    y0 = oracle.y_of(s.dm0)
    with _gpu(s, adjoint=True) as g:
        sv, dP, dy0 = g.adjoint_rk4(s.t0, y0, dt, int(steps[-1]), steps, w, slot=0, bstart=s.nv_dm, checkpoint=5,
                                    want_dy0=True)
    J0, s_fwd = _objective(s, y0, dt, steps, w)
    assert rel(sv, s_fwd) < 1e-12
    n = s.P1.size
    d1 = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * np.abs(s.P1).max()
    d2 = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * np.abs(s.P2).max()
    jp, _ = _objective(s, y0, dt, steps, w, s.P1 + FD_H * d1, s.P2 + FD_H * d2)
    jm, _ = _objective(s, y0, dt, steps, w, s.P1 - FD_H * d1, s.P2 - FD_H * d2)
    fd = (jp - jm) / (2 * FD_H)
    ad = np.vdot(dP[0].reshape(-1), d1).real + np.vdot(dP[1].reshape(-1), d2).real
    dm = rng.standard_normal(s.dm0.shape) + 1j * rng.standard_normal(s.dm0.shape)
    dm = dm.reshape(s.nk, nb_dm, nb_dm)
    dm = 0.5 * (dm + np.conj(np.swapaxes(dm, 1, 2)))
    dy = oracle.y_of(dm.reshape(s.nk, -1)) * 1e-3
    jp, _ = _objective(s, y0 + FD_H * dy, dt, steps, w)
    jm, _ = _objective(s, y0 - FD_H * dy, dt, steps, w)
    fdy = (jp - jm) / (2 * FD_H)
    ady = float(np.dot(dy0, dy))
    print("nb_dm %d window [%d,%d) picture %d: dJ/dP rel %.3g, dJ/dy0 rel %.3g"
          % (nb_dm, bstart, bend, picture, abs(ad - fd) / abs(fd), abs(ady - fdy) / abs(fdy)))
    assert abs(ad - fd) <= TOL * abs(fd)
    assert abs(ady - fdy) <= TOL * abs(fdy)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["nb2_eimp_B", "nb2_schrod", "nb4_eimp_B", "nb2_window"])
def test_double_float_backward_matches_fp64(case, oracle, built):
    """a double-float ("f64x") handle runs the backward pair pass in double-float arithmetic
    (k_adj_pairs_df, gradient kept as double-floats): its dJ/dP and dJ/dy0 equal the FP64 handle's
    (k_adj_pairs) to the forms' accuracy, far inside the adjoint's 1e-5"""
    s = oracle.load(os.path.join(GOLDEN, case))
    rng = np.random.default_rng(5)
    dt = 2.0 * oracle.fs
    steps = np.array([0, 9, 20, 33])
    w = rng.standard_normal(steps.size)
    y0 = oracle.y_of(s.dm0)
    out = {}
    for prec in ("f64", "f64x"):
        with _gpu(s, adjoint=True, precision=prec) as g:
            out[prec] = g.adjoint_rk4(s.t0, y0, dt, int(steps[-1]), steps, w, slot=0, bstart=s.nv_dm, checkpoint=7,
                                      want_dy0=True)
    (s64, dP64, dy64), (sdf, dPdf, dydf) = out["f64"], out["f64x"]
    e_s, e_p, e_y = rel(sdf, s64), rel(dPdf, dP64), rel(dydf, dy64)
    print("%s f64x vs f64 adjoint: S %.3g dJ/dP %.3g dJ/dy0 %.3g" % (case, e_s, e_p, e_y))
    assert e_s < 1e-11 and e_p < 1e-9 and e_y < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["f64", "f64x"])
def test_kept_stages_equal_recomputed_stretches(prec, oracle, built, monkeypatch):
    """the backward pass over stages kept by the forward pass and over stretches recomputed from
    checkpoints (DMD_ADJ_KEEP_ALL=0, 7 steps per stretch) give the same gradients"""
    s = oracle.load(os.path.join(GOLDEN, "nb4_eimp_B"))
    rng = np.random.default_rng(9)
    steps = np.array([0, 9, 20, 33])
    w = rng.standard_normal(steps.size)
    out = {}
    for keep in ("1", "0"):
        monkeypatch.setenv("DMD_ADJ_KEEP_ALL", keep)
        with _gpu(s, adjoint=True, precision=prec) as g:
            out[keep] = g.adjoint_rk4(s.t0, oracle.y_of(s.dm0), 2.0 * oracle.fs, int(steps[-1]), steps, w, slot=0,
                                      bstart=s.nv_dm, checkpoint=7, want_dy0=True)
    assert rel(out["1"][0], out["0"][0]) < 1e-13
    assert rel(out["1"][1], out["0"][1]) < 1e-12
    assert rel(out["1"][2], out["0"][2]) < 1e-12


def _mode_model(oracle, tmp_path, nb=2, nk=60, nsteps=60):
    """a synthetic system whose operators are sum_m theta_m P^(m): 6 phonon modes + impurities"""
    from denmat_dynm_development_gb300.adjoint import ModeScaledRK4
    from denmat_dynm_development_gb300.ldbd_synth import SynthConfig, make_ldbd, mode_operators
    cfg = SynthConfig(nk=nk, nb=nb, seed=11, eimp_sigma_mev=5.0)
    make_ldbd(str(tmp_path), cfg, B_T=(0.3, 0.0, 0.0))
    s = oracle.load(str(tmp_path))
    _, P1m, P2m, Q1, Q2 = mode_operators(cfg)
    P1m = np.concatenate([P1m, Q1[None]])
    P2m = np.concatenate([P2m, Q2[None]])
    # impurity scale 0.2: at the loader's 1e-2 the impurities move S_z by ~1e-6 of itself over this
    # horizon, below what a central difference with h = 1e-4 resolves in FP64
    theta = np.array([1.0, 0.8, 1.3, 1.0, 0.6, 1.1, 0.2])
    steps = np.arange(0, nsteps + 1, 10)
    model = ModeScaledRK4(nk=s.nk, nb_dm=s.nb_dm, bstart=s.bstart, bend=s.bend, e_dm=s.e_dm, k1st=s.k1st,
                          k2nd=s.k2nd, P1_modes=P1m, P2_modes=P2m, prefac_eph=s.prefac_eph, y0=oracle.y_of(s.dm0),
                          dt=2.0 * oracle.fs, nsteps=nsteps, obs_steps=steps, obs=s.smat[:, 2, :], f_obs=s.f_dm,
                          ob_prefac=s.ob_prefac, obs_bstart=s.nv_dm, t0=s.t0, Hcoh=s.Hcoh,
                          picture=s.picture_schrodinger, expt=s.expt, precision="f64", checkpoint=16)
    return s, model, theta, steps


@pytest.mark.gpu
def test_mode_scale_gradient_vs_fd_gpu_and_oracle(oracle, built, tmp_path):
    s, model, theta, steps = _mode_model(oracle, tmp_path)
    w = np.zeros(steps.size)
    w[-1] = 1.0  # J = S_z(t_f)
    sv, grad = model.gradient(theta, w)
    fd = np.zeros(theta.size)
    for m in range(theta.size):
        e = np.zeros(theta.size)
        e[m] = FD_H * theta[m]
        fd[m] = (model.forward(theta + e)[-1] - model.forward(theta - e)[-1]) / (2 * FD_H * theta[m])
    print("dS_z(t_f)/dtheta adjoint", grad, "\n fd", fd)
    assert rel(grad, fd) < TOL
    # the FP64 oracle's forward (the reference's algorithm) for two of the scales
    y0 = oracle.y_of(s.dm0)
    for m in (1, theta.size - 1):
        vals = []
        for sg in (1, -1):
            th = theta.copy()
            th[m] += sg * FD_H * theta[m]
            P1, P2 = model.operators(th)
            so = dataclasses.replace(s, P1=np.ascontiguousarray(P1.reshape(-1)), P2=np.ascontiguousarray(P2.reshape(-1)))
            y, _ = oracle.rk4(so, s.t0, model.dt, model.nsteps, y0)
            vals.append(oracle.measure(so, y, s.t0 + model.nsteps * model.dt)[0])
        fo = (vals[0] - vals[1]) / (2 * FD_H * theta[m])
        print("mode %d: adjoint %.12g oracle fd %.12g" % (m, grad[m], fo))
        assert abs(grad[m] - fo) <= TOL * abs(fo)


@pytest.mark.gpu
def test_autograd_through_fitted_lifetime(oracle, built, tmp_path):
    torch = pytest.importorskip("torch")
    from denmat_dynm_development_gb300.adjoint import sz_trajectory, t1_loglinear
    s, model, theta, steps = _mode_model(oracle, tmp_path, nsteps=80)
    t = steps * model.dt
    th = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    tau = t1_loglinear(t, sz_trajectory(th, model))
    tau.backward()
    g = th.grad.numpy()
    for m in (0, 3, theta.size - 1):
        e = np.zeros(theta.size)
        e[m] = FD_H * theta[m]
        tp = float(t1_loglinear(t, torch.as_tensor(model.forward(theta + e))))
        tm = float(t1_loglinear(t, torch.as_tensor(model.forward(theta - e))))
        fd = (tp - tm) / (2 * FD_H * theta[m])
        print("dT1/dtheta_%d: autograd %.12g fd %.12g" % (m, g[m], fd))
        assert abs(g[m] - fd) <= TOL * abs(fd)


def test_mode_operators_sum_to_the_combined_operators():
    from denmat_dynm_development_gb300.ldbd_synth import SynthConfig, generate_arrays, mode_operators
    cfg = SynthConfig(nk=40, nb=2, seed=5, eimp_sigma_mev=5.0)
    _, P1, P2, Q1, Q2 = generate_arrays(cfg, fold_fraction=None, procs=1)
    _, P1m, P2m, R1, R2 = mode_operators(cfg)
    assert P1m.shape == (cfg.nmodes,) + P1.shape
    assert rel(P1m.sum(0), P1) < 1e-14 and rel(P2m.sum(0), P2) < 1e-14
    np.testing.assert_array_equal(R1, Q1)
    np.testing.assert_array_equal(R2, Q2)


def test_t1_loglinear_recovers_an_exponential():
    torch = pytest.importorskip("torch")
    from denmat_dynm_development_gb300.adjoint import t1_loglinear
    t = np.linspace(0, 10, 21)
    s = torch.tensor(3e-4 * np.exp(-t / 4.5), dtype=torch.float64)
    assert abs(float(t1_loglinear(t, s)) - 4.5) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["f64", "f64x"])
def test_add_operators_equals_a_new_handle(precision, oracle, built):
    """dmd_add_operators (P += scale P_add on the device, stored form rebuilt) gives the RHS of a
    handle created with the shifted operators, and adding the opposite shift restores it."""
    s = oracle.load(os.path.join(GOLDEN, "nb4_eimp_B"))
    rng = np.random.default_rng(2)
    A1 = 1e-2 * (rng.standard_normal(s.P1.shape) + 1j * rng.standard_normal(s.P1.shape)) * np.abs(s.P1).max()
    A2 = 1e-2 * (rng.standard_normal(s.P2.shape) + 1j * rng.standard_normal(s.P2.shape)) * np.abs(s.P2).max()
    y = oracle.y_of(s.dm0)
    t = 17.0 * oracle.fs
    tol = 1e-15 if precision == "f64" else 1e-13
    with _gpu(s, adjoint=True, precision=precision) as g, \
            _gpu(s, P1=s.P1 + 0.3 * A1, P2=s.P2 + 0.3 * A2, precision=precision) as h:
        r0 = g.func(t, y)
        g.add_operators(A1, A2, 0.3)
        assert rel(g.func(t, y), h.func(t, y)) < 10 * tol
        g.add_operators(A1, A2, -0.3)
        assert rel(g.func(t, y), r0) < 10 * tol


@pytest.mark.gpu
def test_streamed_mode_model_matches_the_in_memory_one(oracle, built, tmp_path):
    """StreamedModeScaledRK4 (operator sets regenerated chunk by chunk, one device handle, central
    differences by in-place shifts) gives the in-memory model's gradient, and its own central
    differences agree with it at the adjoint's tolerance."""
    from denmat_dynm_development_gb300 import ldbd_synth as S
    from denmat_dynm_development_gb300.adjoint import StreamedModeScaledRK4
    s, model, theta, steps = _mode_model(oracle, tmp_path)
    cfg = S.SynthConfig(nk=60, nb=2, seed=11, eimp_sigma_mev=5.0)  # _mode_model's system
    w = np.zeros(steps.size)
    w[-1] = 1.0
    _, g_mem = model.gradient(theta, w)
    ms = S.ModeSets(cfg, procs=2)
    assert ms.nparams == theta.size and ms.st.npair == s.npair
    sm = StreamedModeScaledRK4(modes=ms, nk=s.nk, nb_dm=s.nb_dm, bstart=s.bstart, bend=s.bend, e_dm=s.e_dm,
                               k1st=s.k1st, k2nd=s.k2nd, prefac_eph=s.prefac_eph, y0=oracle.y_of(s.dm0),
                               dt=model.dt, nsteps=model.nsteps, obs_steps=steps, obs=s.smat[:, 2, :], f_obs=s.f_dm,
                               ob_prefac=s.ob_prefac, theta=theta, obs_bstart=s.nv_dm, t0=s.t0, Hcoh=s.Hcoh,
                               picture=s.picture_schrodinger, expt=s.expt, precision="f64", checkpoint=16)
    try:
        _, g_st = sm.gradient(w)
        fd = sm.central_differences(w, FD_H)
    finally:
        sm.close()
    print("streamed adjoint", g_st, "\n in-memory", g_mem, "\n fd", fd)
    assert rel(g_st, g_mem) < 1e-10
    assert rel(g_st, fd) < TOL
