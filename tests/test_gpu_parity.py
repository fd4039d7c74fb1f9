"""GPU parity: the CUDA path through the C ABI against the golden fixtures and the oracle.

Tolerances (normwise relative, max|gpu - ref| / max|ref|):
  * RHS (func, evolve_driver, evolve_coh) in FP64: 1e-12 -- the reference forms each P(t)
    element's phase cis(t(e1-e3-e2+e4)) while the GPU factorises it per k, and the pair sums
    run in a different order;
  * RHS in the FP32-pair ("f64x") arithmetic: 1e-11 -- products carry ~2^-47 relative error and
    the scattering-in and scattering-out terms of the finish partly cancel;
  * trajectories (40 RK4 steps, RKF45 to 20 fs): 1e-10 (the bound rho(t) and S(t) are held to).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, FIXED_P_CASES

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def make_gpu(s, precision="f64"):
    from denmat_dynm_development_gb300.dmd import LindbladGPU
    lin = bool(getattr(s, "linear", False))
    g = LindbladGPU(nk=s.nk, nb_dm=s.nb_dm, bstart=s.bstart, bend=s.bend, e_dm=s.e_dm, k1st=s.k1st, k2nd=s.k2nd,
                    P1=s.P1, P2=s.P2, prefac_eph=s.prefac_eph, Hcoh=s.Hcoh, picture=s.picture_schrodinger,
                    expt=s.expt, precision=precision, linear=lin, f_ref=s.f_eq if lin else None)
    if getattr(s, "ddmdt_eq", None) is not None:
        g.set_ddmdt_eq(s.ddmdt_eq)
    return g


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as G
    G.build()


RHS_TOL = {"f64": 1e-12, "f64x": 1e-11}


def cases_for(prec):
    return [(c, prec) for c in FIXED_P_CASES]


ALL = cases_for("f64") + cases_for("f64x")


@pytest.mark.parametrize("case,prec", ALL)
def test_rhs_vs_golden(case, prec, oracle, built):
    d = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(d, "golden.npz")))
    s = oracle.load(d)
    tol = RHS_TOL[prec]
    with make_gpu(s, prec) as gpu:
        for i, t in enumerate(g["rhs_t"]):
            y = g["rhs_y"][i]
            e1 = rel(gpu.func(t, y), g["rhs_dydt"][i])
            e2 = rel(gpu.evolve_driver(t, y), g["rhs_eph"][i])
            print("%s %s t=%g func %.3g eph %.3g" % (case, prec, t, e1, e2))
            assert e1 < tol and e2 < tol
            if np.abs(g["rhs_coh"][i]).max() > 0:
                assert rel(gpu.evolve_coh(t, y), g["rhs_coh"][i]) < 1e-12
            # exact Hermiticity of the scattering term (c + c^dagger, evolve_eph.cpp:151)
            e = gpu.evolve_driver(t, y).view(np.complex128).reshape(s.nk, s.nb_dm, s.nb_dm)
            np.testing.assert_array_equal(e, np.conj(np.swapaxes(e, 1, 2)))


@pytest.mark.parametrize("case,prec", ALL)
def test_rk4_vs_golden(case, prec, oracle, built):
    d = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(d, "golden.npz")))
    s = oracle.load(d)
    with make_gpu(s, prec) as gpu:
        gpu.set_state(s.t0, oracle.y_of(s.dm0))
        gpu.set_observable(0, s.smat[:, 2, :], s.f_dm, s.ob_prefac)
        rec = []
        for _ in range(8):
            gpu.rk4(1.0 * oracle.fs, 5)
            t, _ = gpu.get_state()
            tot, amp = gpu.measure(0, s.nv_dm)
            rec.append((t, tot, amp))
        t, y = gpu.get_state()
        assert rel(y, g["rk4_y"]) < 1e-10
        rec = np.array(rec)
        ref = g["rk4_sz"][1:]
        assert rel(rec[:, 0], ref[:, 0]) < 1e-14
        assert rel(rec[:, 1], ref[:, 1]) < 1e-10
        assert rel(rec[:, 2], ref[:, 2]) < 1e-10


@pytest.mark.parametrize("case", FIXED_P_CASES)
def test_host_rk4_over_callback_vs_golden(case, oracle, built):
    """dmdh_rk4_func (the host drives RK4 through the GSL-callback entry, 4 dmd_func calls per step)
    reaches the reference's RK4 state after 40 steps, like the device-resident loop"""
    from denmat_dynm_development_gb300 import host as HL
    d = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(d, "golden.npz")))
    s = oracle.load(d)
    with make_gpu(s, "f64") as gpu:
        y = np.ascontiguousarray(oracle.y_of(s.dm0), dtype=np.float64).copy()
        work = np.zeros(5 * y.size)
        HL.rk4_func(gpu, s.t0, 1.0 * oracle.fs, 40, y, work)
        assert rel(y, g["rk4_y"]) < 1e-10
        gpu.set_state(s.t0, oracle.y_of(s.dm0))
        gpu.rk4(1.0 * oracle.fs, 40)
        _, yd = gpu.get_state()
        assert rel(y, yd) < 1e-13


@pytest.mark.parametrize("case,prec", ALL)
def test_rkf45_vs_golden(case, prec, oracle, built):
    """DMD's evolve_gsl loop: one driver_apply per output interval (DensityMatrix_Dynamics.h:210-223)."""
    d = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(d, "golden.npz")))
    s = oracle.load(d)
    with make_gpu(s, prec) as gpu:
        gpu.set_state(s.t0, oracle.y_of(s.dm0))
        gpu.set_observable(0, s.smat[:, 2, :], s.f_dm, s.ob_prefac)
        hs = s.ode["hstart"]
        ti = s.t0
        tcur = s.t0
        sz, nf = [], []
        while tcur < s.tend:
            ti += s.tstep
            hs, n = gpu.rkf45_apply(ti, hs, s.ode["hmin"], s.ode["hmax"], s.ode["epsabs"], 0.0)
            tcur, _ = gpu.get_state()
            sz.append(gpu.measure(0, s.nv_dm)[0])
            nf.append(n)
        _, y = gpu.get_state()
        assert rel(y, g["gsl_y"]) < 1e-10
        assert rel(np.array(sz), g["gsl_sz"][1:, 1]) < 1e-10
        np.testing.assert_array_equal(np.array(nf), g["gsl_ncalls"])


@pytest.mark.parametrize("case", FIXED_P_CASES)
def test_euler_vs_oracle(case, oracle, built):
    d = os.path.join(GOLDEN, case)
    s = oracle.load(d)
    y0 = oracle.y_of(s.dm0)
    with make_gpu(s) as gpu:
        gpu.set_state(s.t0, y0)
        gpu.euler(0.5 * oracle.fs, 6)
        _, y = gpu.get_state()
    yr = oracle.euler(s, s.t0, 0.5 * oracle.fs, 6, y0)
    assert rel(y, yr) < 1e-12


@pytest.mark.parametrize("prec", ["f64", "f64x"])
def test_larger_random_case_vs_oracle(prec, oracle, built, tmp_path):
    """nk=500 Si-like workload (about 70k pairs) with e-imp and a B field."""
    from denmat_dynm_development_gb300.ldbd_synth import SynthConfig, make_ldbd
    cfg = SynthConfig(nk=500, nb=2, seed=3, eimp_sigma_mev=5.0)
    make_ldbd(str(tmp_path), cfg, B_T=(1.0, 0.0, 0.0), eimp_fraction=1e-2)
    s = oracle.load(str(tmp_path))
    rng = np.random.default_rng(5)
    with make_gpu(s, prec) as gpu:
        for t in (0.0, 11.0 * oracle.fs, 4000.0 * oracle.fs):
            dm = s.dm0 + 1e-3 * (rng.standard_normal(s.dm0.shape) + 1j * rng.standard_normal(s.dm0.shape))
            dm = dm.reshape(s.nk, s.nb_dm, s.nb_dm)
            dm = 0.5 * (dm + np.conj(np.swapaxes(dm, 1, 2)))
            y = oracle.y_of(dm.reshape(s.nk, -1))
            err = rel(gpu.func(t, y), oracle.rhs(s, t, y))
            print("nk500 %s t=%g rel err %.3g" % (prec, t, err))
            assert err < RHS_TOL[prec]


@pytest.mark.parametrize("prec", ["f64", "f64x"])
def test_irregular_pairs_vs_oracle(prec, oracle, built):
    """Duplicated pairs, pairs stored with k1 > k2 (no reverse term) and diagonal pairs, as the
    reference's loop accepts them (evolve_eph.cpp:49-106)."""
    d = os.path.join(GOLDEN, "nb2_eimp_B")
    s0 = oracle.load(d)
    rng = np.random.default_rng(9)
    n = s0.npair
    nb4 = 16
    P1 = s0.P1.reshape(n, nb4)
    P2 = s0.P2.reshape(n, nb4)
    dup = rng.choice(n, 40, replace=False)
    swp = rng.choice(n, 60, replace=False)
    k1 = np.concatenate([s0.k1st, s0.k1st[dup], s0.k2nd[swp], np.arange(5, dtype=np.uint64)])
    k2 = np.concatenate([s0.k2nd, s0.k2nd[dup], s0.k1st[swp], np.arange(5, dtype=np.uint64)])
    Q1 = np.concatenate([P1, 0.5 * P1[dup], 0.3 * P2[swp], P1[:5]])
    Q2 = np.concatenate([P2, 0.7 * P2[dup], 0.2 * P1[swp], P2[:5]])
    s = oracle.from_arrays(nk=s0.nk, nb_dm=s0.nb_dm, bstart=s0.bstart, bend=s0.bend, e_dm=s0.e_dm, f_dm=s0.f_dm,
                           k1st=k1, k2nd=k2, P1=Q1.reshape(-1), P2=Q2.reshape(-1), prefac_eph=s0.prefac_eph,
                           dm0=s0.dm0, Hcoh=s0.Hcoh)
    y = oracle.y_of(s.dm0)
    t = 9.0 * oracle.fs
    with make_gpu(s, prec) as gpu:
        err = rel(gpu.func(t, y), oracle.rhs(s, t, y))
    assert err < RHS_TOL[prec]


@pytest.mark.parametrize("prec", ["f64", "f64x"])
def test_nb4_larger_vs_oracle(prec, oracle, built, tmp_path):
    """nb = 4 (four lanes share a pair, 8-column blocks) on a larger random case."""
    from denmat_dynm_development_gb300.ldbd_synth import SynthConfig, make_ldbd
    cfg = SynthConfig(nk=120, nb=4, seed=4, eimp_sigma_mev=5.0)
    make_ldbd(str(tmp_path), cfg, B_T=(0.0, 0.7, 0.0), eimp_fraction=1e-2)
    s = oracle.load(str(tmp_path))
    y = oracle.y_of(s.dm0)
    with make_gpu(s, prec) as gpu:
        t = 250.0 * oracle.fs
        err = rel(gpu.func(t, y), oracle.rhs(s, t, y))
        print("nb4 %s npair=%d rel err %.3g" % (prec, s.npair, err))
        assert err < RHS_TOL[prec]
        gpu.set_state(s.t0, y)
        gpu.rk4(2.0 * oracle.fs, 10)
        _, yg = gpu.get_state()
    yr, _ = oracle.rk4(s, s.t0, 2.0 * oracle.fs, 10, y)
    assert rel(yg, yr) < 1e-10


@pytest.mark.parametrize("case", ["nb2_carrier_eq", "nb2_holes_eq"])
def test_equilibrium_drift_on_gpu(case, built):
    """dmdh_prepare computes compute_ddmdt_eq's drift with the GPU RHS (evolve_eph.cpp:3-19) and
    installs it; the result matches the reference's drift and the RHS with it subtracted."""
    from denmat_dynm_development_gb300.host import System
    d = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(d, "golden.npz")))
    s = System(d)
    with s.gpu("f64") as gpu:
        i = s.info
        y = np.zeros((s.nk, s.nb_dm, s.nb_dm), np.complex128)
        idx = np.arange(s.nb_dm)
        y[:, idx, idx] = s.f_eq
        # with the drift installed, diag(f_eq) is stationary under the scattering term at t = 0
        eph = gpu.evolve_driver(0.0, y.reshape(s.nk, -1).view(np.float64).reshape(-1).copy())
        scale = np.abs(g["ddmdt_eq"]).max()
        assert np.abs(eph).max() < 1e-12 * scale
        for k, t in enumerate(g["rhs_t"]):
            assert rel(gpu.func(t, g["rhs_y"][k]), g["rhs_dydt"][k]) < 1e-12
        assert i.ddmdteq == 1


@pytest.mark.parametrize("prec", ["f64", "f64x"])
def test_t1_from_gpu_trajectory(prec, oracle, built):
    """T1 (the fit.py restatement) from the GPU RK4 trajectory against the oracle's: S(t) within the
    trajectory bound 1e-10, and the least-squares lifetime converged to machine precision (tau_conv)
    within 1e-10 -- the bound the FP64 path is held to for rho(t), S(t) and the fitted T1/T2. The
    fit.py-faithful tau_lsq / tau_cf stop at leastsq's xtol (~1.5e-8 on beta) and are compared at
    the tolerance that xtol allows."""
    from denmat_dynm_development_gb300.t1fit import fit_t1
    s = oracle.load(os.path.join(GOLDEN, "nb2_carrier_eq"))
    h, nsteps, every = 2.0 * oracle.fs, 1500, 50
    y0 = oracle.y_of(s.dm0)
    _, rec_o = oracle.rk4(s, s.t0, h, nsteps, y0, every=every)
    with make_gpu(s, prec) as gpu:
        gpu.set_state(s.t0, y0)
        gpu.set_observable(0, s.smat[:, 2, :], s.f_dm, s.ob_prefac)
        rec = []
        for _ in range(nsteps // every):
            gpu.rk4(h, every)
            t, _ = gpu.get_state()
            rec.append((t,) + gpu.measure(0, s.nv_dm))
    rec = np.array(rec)
    assert rel(rec[:, 1], rec_o[:, 1]) < 1e-10
    fo = fit_t1(rec_o[:, 0], rec_o[:, 1])
    fg = fit_t1(rec[:, 0], rec[:, 1])
    err = abs(fg.tau_conv - fo.tau_conv) / abs(fo.tau_conv)
    print("%s: T1 oracle %.15g ps gpu %.15g ps (converged fit), rel err %.3g; S(t) rel err %.3g"
          % (prec, fo.tau_conv, fg.tau_conv, err, rel(rec[:, 1], rec_o[:, 1])))
    # the synthetic P follows the initializer's smeared-delta construction without detailed balance,
    # so |S| need not decay; the fit is still a well-defined function of the trajectory
    assert np.isfinite(fo.tau_conv) and np.isfinite(fg.tau_conv)
    assert err < 1e-10
    # leastsq / curve_fit stop at xtol ~1.5e-8 on beta, which moves their answers by up to ~1e-7
    assert abs(fg.tau_lsq - fo.tau_lsq) / abs(fo.tau_lsq) < 1e-6
    assert abs(fg.tau_cf - fo.tau_cf) / abs(fo.tau_cf) < 1e-6


@pytest.mark.parametrize("prec", ["f64", "f64x"])
def test_non_hermitian_state_vs_oracle(prec, oracle, built):
    """func on a state that is not Hermitian (the GSL callback accepts any y): the contraction runs
    its anti-Hermitian pass, and a Hermitian state right after must not see a stale flag."""
    s = oracle.load(os.path.join(GOLDEN, "nb2_eimp_B"))
    rng = np.random.default_rng(21)
    t = 13.0 * oracle.fs
    dm = s.dm0 + 1e-3 * (rng.standard_normal(s.dm0.shape) + 1j * rng.standard_normal(s.dm0.shape))
    y_nh = oracle.y_of(dm)
    d = dm.reshape(s.nk, s.nb_dm, s.nb_dm)
    y_h = oracle.y_of((0.5 * (d + np.conj(np.swapaxes(d, 1, 2)))).reshape(s.nk, -1))
    with make_gpu(s, prec) as gpu:
        for y in (y_nh, y_h, y_nh):
            err = rel(gpu.func(t, y), oracle.rhs(s, t, y))
            assert err < RHS_TOL[prec], err


# Reduced-precision forms (P stored FP32 or bf16 hi+lo, FP32 products): rho enters as its deviation
# from f_ref = f_dm, the contraction of diag(f_ref) is formed once in FP64. Tolerances, normwise
# relative to the oracle's RHS: FP32 storage 1e-6, bf16 hi+lo (16 significant bits) 1e-5; the fitted
# T1 within 1e-4 relative of the FP64 oracle (the target of the reduced-precision forms).
LOWP_TOL = {"f32": 1e-6, "bf16x2": 1e-5}
# the tensor-core batched form rounds the coordinates of rho to bf16 hi + lo as well (16 significant
# bits on both operands of every product)
TC_TOL = 2e-5


def make_gpu_lowp(s, prec, with_ref=True, nrhs=1):
    from denmat_dynm_development_gb300.dmd import LindbladGPU
    lin = bool(getattr(s, "linear", False))
    g = LindbladGPU(nk=s.nk, nb_dm=s.nb_dm, bstart=s.bstart, bend=s.bend, e_dm=s.e_dm, k1st=s.k1st, k2nd=s.k2nd,
                    P1=s.P1, P2=s.P2, prefac_eph=s.prefac_eph, Hcoh=s.Hcoh, picture=s.picture_schrodinger,
                    expt=s.expt, precision=prec, linear=lin,
                    f_ref=s.f_eq if lin else (s.f_dm if with_ref else None), nrhs=nrhs)
    if getattr(s, "ddmdt_eq", None) is not None:
        g.set_ddmdt_eq(s.ddmdt_eq)
    return g


@pytest.mark.parametrize("prec", ["f32", "bf16x2"])
@pytest.mark.parametrize("case", ["nb2_eimp_B", "nb2_window", "nb2_carrier_eq", "nb4_eimp_B", "nb2_linear", "nb4_linear"])
def test_lowp_rhs_vs_golden(case, prec, oracle, built):
    d = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(d, "golden.npz")))
    s = oracle.load(d)
    with make_gpu_lowp(s, prec) as gpu:
        for i, t in enumerate(g["rhs_t"]):
            e = rel(gpu.func(t, g["rhs_y"][i]), g["rhs_dydt"][i])
            print("%s %s t=%g rel err %.3g" % (case, prec, t, e))
            assert e < LOWP_TOL[prec]


def test_lowp_without_reference_occupations(oracle, built):
    """f_ref omitted: the deviation is taken from zero occupations (still correct, less accurate)."""
    d = os.path.join(GOLDEN, "nb2_eimp_B")
    g = dict(np.load(os.path.join(d, "golden.npz")))
    s = oracle.load(d)
    with make_gpu_lowp(s, "f32", with_ref=False) as gpu:
        e = rel(gpu.func(g["rhs_t"][1], g["rhs_y"][1]), g["rhs_dydt"][1])
        print("f32 without f_ref: rel err %.3g" % e)
        assert e < 1e-3


@pytest.mark.parametrize("prec", ["f32", "bf16x2"])
def test_lowp_t1_vs_oracle(prec, oracle, built):
    from denmat_dynm_development_gb300.t1fit import fit_t1
    s = oracle.load(os.path.join(GOLDEN, "nb2_carrier_eq"))
    h, nsteps, every = 2.0 * oracle.fs, 1500, 50
    y0 = oracle.y_of(s.dm0)
    _, rec_o = oracle.rk4(s, s.t0, h, nsteps, y0, every=every)
    with make_gpu_lowp(s, prec) as gpu:
        gpu.set_state(s.t0, y0)
        gpu.set_observable(0, s.smat[:, 2, :], s.f_dm, s.ob_prefac)
        rec = []
        for _ in range(nsteps // every):
            gpu.rk4(h, every)
            t, _ = gpu.get_state()
            rec.append((t,) + gpu.measure(0, s.nv_dm))
    rec = np.array(rec)
    es = rel(rec[:, 1], rec_o[:, 1])
    fo, fg = fit_t1(rec_o[:, 0], rec_o[:, 1]), fit_t1(rec[:, 0], rec[:, 1])
    et = abs(fg.tau_conv - fo.tau_conv) / abs(fo.tau_conv)
    print("%s: S(t) rel err %.3g, T1 %.10g vs %.10g ps (converged fit), rel err %.3g"
          % (prec, es, fg.tau_conv, fo.tau_conv, et))
    assert et < 1e-4


def _herm_states(s, n, seed, scale=1e-3):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        d = s.dm0 + scale * (rng.standard_normal(s.dm0.shape) + 1j * rng.standard_normal(s.dm0.shape))
        d = d.reshape(s.nk, s.nb_dm, s.nb_dm)
        d = 0.5 * (d + np.conj(np.swapaxes(d, 1, 2)))
        out.append(np.ascontiguousarray(d.reshape(s.nk, -1)).view(np.float64).reshape(-1))
    return out


def _tensor_core_form(s, prec):
    """the batched form runs on the tensor cores for nb = 2 and nb = 4 with bf16 hi + lo storage"""
    return prec == "bf16x2" and s.bend - s.bstart in (2, 4) and os.environ.get("DMD_BATCH_TC", "1") != "0"


@pytest.mark.parametrize("prec", ["f32", "bf16x2"])
@pytest.mark.parametrize("case", ["nb2_eimp_B", "nb4_eimp_B", "nb2_linear", "nb4_linear", "nb2_carrier_eq",
                                  "nb2_window"])
def test_batched_states_vs_oracle(case, prec, oracle, built):
    """Batched form: 7 states share P (bf16 hi + lo: the tensor-core contraction; else
    RW states per warp on the CUDA cores, the last group short). Every state's RHS matches the oracle
    at the reduced-precision tolerance; 20 RK4 steps of the batch change every state as 20 oracle
    steps do, to that tolerance; the CUDA-core batch also matches each state stepped alone."""
    s = oracle.load(os.path.join(GOLDEN, case))
    R = 7
    ys = _herm_states(s, R, 31)
    t = 41.0 * oracle.fs
    h = 2.0 * oracle.fs
    tc = _tensor_core_form(s, prec)
    tol = TC_TOL if tc else LOWP_TOL[prec]
    with make_gpu_lowp(s, prec, nrhs=R) as gb:
        out = gb.func(t, np.concatenate(ys)).reshape(R, -1)
        for q in range(R):
            e = rel(out[q], oracle.rhs(s, t, ys[q]))
            assert e < tol, (q, e)
        gb.set_state(s.t0, np.concatenate(ys))
        gb.rk4(h, 20)
        _, yb = gb.get_state()
        yb = yb.reshape(R, -1)
        gb.set_observable(0, s.smat[:, 2, :], s.f_dm, s.ob_prefac)
        tot, _ = gb.measure_batch(0, s.nv_dm)
    for q in (0, 3, R - 1):
        yo, _ = oracle.rk4(s, s.t0, h, 20, ys[q])
        e = rel(yb[q] - ys[q], yo - ys[q])
        print("%s %s state %d: 20-step change rel err %.3g" % (case, prec, q, e))
        assert e < 3 * tol
        with make_gpu_lowp(s, prec) as g1:
            g1.set_state(s.t0, ys[q])
            g1.rk4(h, 20)
            _, y1 = g1.get_state()
            g1.set_observable(0, s.smat[:, 2, :], s.f_dm, s.ob_prefac)
            t1, _ = g1.measure(0, s.nv_dm)
        if not tc:
            # the batch and the single state sum in different atomic orders: FP32-level differences
            # of the RHS, integrated over 20 steps
            assert rel(yb[q], y1) < 1e-10
        assert abs(tot[q] - t1) <= 1e-5 * abs(t1)


def test_batched_tensor_core_many_states(oracle, built, tmp_path, monkeypatch):
    """Tensor-core batched form on a larger random case (nk = 500, about 70k pairs, tiles spanning
    many column groups) with 130 states: two state blocks of 128, the second nearly empty. Every
    checked state matches the oracle; the whole batch matches the CUDA-core batched form
    (DMD_BATCH_TC=0); a batch holding non-Hermitian states runs the anti-Hermitian pass."""
    from denmat_dynm_development_gb300.ldbd_synth import SynthConfig, make_ldbd
    cfg = SynthConfig(nk=500, nb=2, seed=3, eimp_sigma_mev=5.0)
    make_ldbd(str(tmp_path), cfg, B_T=(1.0, 0.0, 0.0), eimp_fraction=1e-2)
    s = oracle.load(str(tmp_path))
    R = 130
    ys = _herm_states(s, R, 12)
    t = 11.0 * oracle.fs
    with make_gpu_lowp(s, "bf16x2", nrhs=R) as gb:
        out_tc = gb.func(t, np.concatenate(ys)).reshape(R, -1)
    monkeypatch.setenv("DMD_BATCH_TC", "0")
    with make_gpu_lowp(s, "bf16x2", nrhs=R) as gc:
        out_cc = gc.func(t, np.concatenate(ys)).reshape(R, -1)
    monkeypatch.delenv("DMD_BATCH_TC")
    for q in (0, 1, 64, 127, 128, 129):
        e = rel(out_tc[q], oracle.rhs(s, t, ys[q]))
        print("nk500 state %d: tensor-core rel err %.3g" % (q, e))
        assert e < TC_TOL
    for q in range(R):
        assert rel(out_tc[q], out_cc[q]) < TC_TOL + LOWP_TOL["bf16x2"], q
    # non-Hermitian states in the batch (the GSL callback accepts any y)
    rng = np.random.default_rng(4)
    nh = [y + 1e-3 * rng.standard_normal(y.shape) for y in ys[:3]]
    with make_gpu_lowp(s, "bf16x2", nrhs=3) as gb:
        for batch in (nh, ys[:3], nh):
            out = gb.func(t, np.concatenate(batch)).reshape(3, -1)
            for q in range(3):
                assert rel(out[q], oracle.rhs(s, t, batch[q])) < TC_TOL, q


def test_batched_tensor_core_nb4_many_states(oracle, built, tmp_path, monkeypatch):
    """Tensor-core batched form for nb = 4 (tiles of 4 rows, column groups of 2) on a random case
    (nk = 240, spin-split pairs of bands) with 129 states: every checked state matches the oracle and
    the whole batch matches the CUDA-core batched form (DMD_BATCH_TC=0); 10 RK4 steps of the batch
    change the states as the oracle's steps do."""
    from denmat_dynm_development_gb300.ldbd_synth import SynthConfig, make_ldbd
    cfg = SynthConfig(nk=240, nb=4, seed=8, eimp_sigma_mev=5.0)
    make_ldbd(str(tmp_path), cfg, B_T=(0.0, 0.0, 0.5), eimp_fraction=1e-2)
    s = oracle.load(str(tmp_path))
    R = 129
    ys = _herm_states(s, R, 21)
    t = 7.0 * oracle.fs
    with make_gpu_lowp(s, "bf16x2", nrhs=R) as gb:
        out_tc = gb.func(t, np.concatenate(ys)).reshape(R, -1)
        h = 2.0 * oracle.fs
        gb.set_state(s.t0, np.concatenate(ys))
        gb.rk4(h, 10)
        _, yb = gb.get_state()
        yb = yb.reshape(R, -1)
    monkeypatch.setenv("DMD_BATCH_TC", "0")
    with make_gpu_lowp(s, "bf16x2", nrhs=R) as gc:
        out_cc = gc.func(t, np.concatenate(ys)).reshape(R, -1)
    monkeypatch.delenv("DMD_BATCH_TC")
    for q in (0, 77, 127, 128):
        e = rel(out_tc[q], oracle.rhs(s, t, ys[q]))
        print("nb4 nk240 state %d: tensor-core rel err %.3g" % (q, e))
        assert e < TC_TOL
    for q in range(R):
        assert rel(out_tc[q], out_cc[q]) < TC_TOL + LOWP_TOL["bf16x2"], q
    for q in (0, 128):
        yo, _ = oracle.rk4(s, s.t0, h, 10, ys[q])
        e = rel(yb[q] - ys[q], yo - ys[q])
        print("nb4 nk240 state %d: 10-step change rel err %.3g" % (q, e))
        assert e < 3 * TC_TOL


def test_batched_tensor_core_irregular_pairs(oracle, built):
    """Duplicated pairs (two operators in one block entry), pairs stored with k1 > k2 (no reverse
    term) and diagonal pairs through the tensor-core batched form."""
    d = os.path.join(GOLDEN, "nb2_eimp_B")
    s0 = oracle.load(d)
    rng = np.random.default_rng(9)
    n = s0.npair
    P1 = s0.P1.reshape(n, 16)
    P2 = s0.P2.reshape(n, 16)
    dup = rng.choice(n, 40, replace=False)
    swp = rng.choice(n, 60, replace=False)
    k1 = np.concatenate([s0.k1st, s0.k1st[dup], s0.k2nd[swp], np.arange(5, dtype=np.uint64)])
    k2 = np.concatenate([s0.k2nd, s0.k2nd[dup], s0.k1st[swp], np.arange(5, dtype=np.uint64)])
    Q1 = np.concatenate([P1, 0.5 * P1[dup], 0.3 * P2[swp], P1[:5]])
    Q2 = np.concatenate([P2, 0.7 * P2[dup], 0.2 * P1[swp], P2[:5]])
    s = oracle.from_arrays(nk=s0.nk, nb_dm=s0.nb_dm, bstart=s0.bstart, bend=s0.bend, e_dm=s0.e_dm, f_dm=s0.f_dm,
                           k1st=k1, k2nd=k2, P1=Q1.reshape(-1), P2=Q2.reshape(-1), prefac_eph=s0.prefac_eph,
                           dm0=s0.dm0, Hcoh=s0.Hcoh)
    ys = _herm_states(s, 4, 8)
    t = 9.0 * oracle.fs
    with make_gpu_lowp(s, "bf16x2", nrhs=4) as gb:
        out = gb.func(t, np.concatenate(ys)).reshape(4, -1)
    for q in range(4):
        assert rel(out[q], oracle.rhs(s, t, ys[q])) < TC_TOL, q


def test_batched_tensor_core_t1_vs_oracle(oracle, built):
    """T1 fitted from a state of a tensor-core batch (3 states, 1500 RK4 steps) within 1e-4 of the
    FP64 oracle's, the target of the reduced-precision forms."""
    from denmat_dynm_development_gb300.t1fit import fit_t1
    s = oracle.load(os.path.join(GOLDEN, "nb2_carrier_eq"))
    h, nsteps, every = 2.0 * oracle.fs, 1500, 50
    y0 = oracle.y_of(s.dm0)
    _, rec_o = oracle.rk4(s, s.t0, h, nsteps, y0, every=every)
    ys = [y0] + _herm_states(s, 2, 17)
    with make_gpu_lowp(s, "bf16x2", nrhs=3) as gb:
        gb.set_state(s.t0, np.concatenate(ys))
        gb.set_observable(0, s.smat[:, 2, :], s.f_dm, s.ob_prefac)
        rec = []
        for _ in range(nsteps // every):
            gb.rk4(h, every)
            t, _ = gb.get_state()
            tot, _ = gb.measure_batch(0, s.nv_dm)
            rec.append((t, tot[0]))
    rec = np.array(rec)
    fo, fg = fit_t1(rec_o[:, 0], rec_o[:, 1]), fit_t1(rec[:, 0], rec[:, 1])
    et = abs(fg.tau_conv - fo.tau_conv) / abs(fo.tau_conv)
    print("tensor-core batch: S(t) rel err %.3g, T1 %.10g vs %.10g ps (converged fit), rel err %.3g"
          % (rel(rec[:, 1], rec_o[:, 1]), fg.tau_conv, fo.tau_conv, et))
    assert et < 1e-4


@pytest.mark.parametrize("prec,nrhs", [("f64", 1), ("f64x", 1), ("f32", 5), ("bf16x2", 5)])
def test_autotune_keeps_the_results(prec, nrhs, oracle, built):
    """dmd_autotune times the compiled contraction shapes and keeps the fastest: the RHS stays the
    oracle's (the shapes differ only in summation order), the state is untouched, and stepping
    afterwards (a new captured graph) works."""
    s = oracle.load(os.path.join(GOLDEN, "nb2_eimp_B"))
    ys = _herm_states(s, nrhs, 5)
    t = 17.0 * oracle.fs
    mk = (lambda: make_gpu(s, prec)) if nrhs == 1 else (lambda: make_gpu_lowp(s, prec, nrhs=nrhs))
    tol = RHS_TOL[prec] if nrhs == 1 else (TC_TOL if prec == "bf16x2" else LOWP_TOL[prec])
    shapes = ((0, 1, 2, 3, 4) if prec == "f64x" else (0, 1, 2, 3)) if nrhs == 1 else \
        ((4, 3, 2) if prec == "bf16x2" else (4, 8))
    with mk() as g:
        y = np.concatenate(ys)
        g.set_state(s.t0, y)
        g.rk4(1.0 * oracle.fs, 2)
        _, ya = g.get_state()
        c = g.autotune(2)
        assert c in shapes
        _, yb = g.get_state()
        np.testing.assert_array_equal(ya, yb)
        out = g.func(t, y).reshape(nrhs, -1)
        for q in range(nrhs):
            assert rel(out[q], oracle.rhs(s, t, ys[q])) < tol
        g.rk4(1.0 * oracle.fs, 2)


def test_group_steps_members_as_when_alone(oracle, built):
    """dmd_group_rk4: three handles with different P sets and forms (f64x nb = 2, f64x nb = 4, a
    tensor-core batch of 3) advanced by one graph per step match the same handles stepped alone."""
    from denmat_dynm_development_gb300.dmd import Group
    sa = oracle.load(os.path.join(GOLDEN, "nb2_eimp_B"))
    sb = oracle.load(os.path.join(GOLDEN, "nb4_eimp_B"))
    ya, yb = oracle.y_of(sa.dm0), oracle.y_of(sb.dm0)
    yc = np.concatenate(_herm_states(sa, 3, 9))
    h = 2.0 * oracle.fs

    def handles():
        return [make_gpu(sa, "f64x"), make_gpu(sb, "f64x"), make_gpu_lowp(sa, "bf16x2", nrhs=3)]

    alone = []
    for g, y in zip(handles(), (ya, yb, yc)):
        with g:
            g.set_state(sa.t0, y)
            g.rk4(h, 12)
            alone.append(g.get_state())
    hs = handles()
    try:
        for g, y in zip(hs, (ya, yb, yc)):
            g.set_state(sa.t0, y)
        with Group(hs) as grp:
            grp.rk4(h, 5)
            grp.rk4(h, 7)
        for g, (t1, y1) in zip(hs, alone):
            t2, y2 = g.get_state()
            assert abs(t2 - t1) <= 1e-12 * abs(t1)
            assert rel(y2, y1) < 1e-12
    finally:
        for g in hs:
            g.close()


def _write_c128(path, a):
    np.ascontiguousarray(a, dtype=np.complex128).tofile(str(path))
    return str(path)


@pytest.mark.parametrize("case,prec,nrhs", [("nb2_eimp_B", "f64x", 1), ("nb2_eimp_B", "bf16x2", 1),
                                            ("nb4_eimp_B", "f64x", 1), ("nb2_linear", "f32", 1),
                                            ("nb2_eimp_B", "f32", 3)])
@pytest.mark.parametrize("chunk", [None, "7"])
def test_create_from_files_matches_arrays(case, prec, nrhs, chunk, oracle, built, tmp_path, monkeypatch):
    """dmd_create_from_files streams DMD's operator files (here with additive operators scaled by
    add_scale) through pinned chunks into the device conversion; the handle equals one created from
    the same arrays (the deviation forms fold diag(f_ref) with atomics: rounding-level differences),
    also when the files go through in chunks of 7 pairs."""
    from denmat_dynm_development_gb300.dmd import LindbladGPU
    s = oracle.load(os.path.join(GOLDEN, case))
    if chunk:
        monkeypatch.setenv("DMD_FILL_CHUNK", chunk)
    rng = np.random.default_rng(2)
    A1 = (rng.standard_normal(s.P1.size) + 1j * rng.standard_normal(s.P1.size)) * np.abs(s.P1).max()
    A2 = (rng.standard_normal(s.P2.size) + 1j * rng.standard_normal(s.P2.size)) * np.abs(s.P2).max()
    files = [_write_c128(tmp_path / n, a) for n, a in (("P1.bin", s.P1), ("P2.bin", s.P2), ("A1.bin", A1),
                                                      ("A2.bin", A2))]
    lin = bool(getattr(s, "linear", False))
    kw = dict(nk=s.nk, nb_dm=s.nb_dm, bstart=s.bstart, bend=s.bend, e_dm=s.e_dm, k1st=s.k1st, k2nd=s.k2nd,
              prefac_eph=s.prefac_eph, Hcoh=s.Hcoh, picture=s.picture_schrodinger, expt=s.expt, precision=prec,
              linear=lin, nrhs=nrhs, f_ref=(s.f_eq if lin else s.f_dm) if prec in ("f32", "bf16x2") else None)
    if lin:  # the linearized form takes no additive operators
        files = files[:2]
        arrays = dict(P1=s.P1, P2=s.P2)
    else:
        arrays = dict(P1=s.P1, P2=s.P2, P1_add=A1, P2_add=A2, add_scale=0.3)
        kw["add_scale"] = 0.3
    ys = np.concatenate(_herm_states(s, nrhs, 4))
    t = 23.0 * oracle.fs
    with LindbladGPU(**kw, **{k: v for k, v in arrays.items() if k != "add_scale"}) as ga:
        ra = ga.func(t, ys)
    with LindbladGPU(P1=None, P2=None, P_files=files, **kw) as gf:
        rf = gf.func(t, ys)
    tol = 1e-15 if prec in ("f64", "f64x") else 1e-12
    assert rel(rf, ra) <= tol



def write_sparse(prefix, P, nb4, rng):
    """DMD's sparse operator files: nonzeros of each pair in a random order"""
    n2 = int(round(nb4 ** 0.5))
    P = np.asarray(P, np.complex128).reshape(-1, nb4)
    ns, sv, si, sj = [], [], [], []
    for row in P:
        nz = np.nonzero(row)[0]
        nz = nz[rng.permutation(nz.size)]
        ns.append(nz.size)
        sv.append(row[nz])
        si.append(nz // n2)
        sj.append(nz % n2)
    np.array(ns, np.int32).tofile(prefix + "_ns.bin")
    np.concatenate(sv).astype(np.complex128).tofile(prefix + "_s.bin")
    np.concatenate(si).astype(np.int32).tofile(prefix + "_i.bin")
    np.concatenate(sj).astype(np.int32).tofile(prefix + "_j.bin")
    return prefix


@pytest.mark.parametrize("prec", ["f64x", "bf16x2"])
def test_create_from_sparse_files_matches_dense(prec, oracle, built, tmp_path, monkeypatch):
    """DMD's sparse operator input (alg.Pin_is_sparse): operators with structural zeros written as
    per-pair (count, values, row, column) files in a random element order, streamed in chunks of 5
    pairs, equal the dense operators."""
    from denmat_dynm_development_gb300.dmd import LindbladGPU
    s = oracle.load(os.path.join(GOLDEN, "nb2_eimp_B"))
    rng = np.random.default_rng(8)
    P1 = s.P1.copy().reshape(-1, 16)
    P2 = s.P2.copy().reshape(-1, 16)
    P1[rng.random(P1.shape) < 0.4] = 0  # structural zeros
    P2[rng.random(P2.shape) < 0.4] = 0
    P1[3] = 0  # an empty operator
    monkeypatch.setenv("DMD_FILL_CHUNK", "5")
    sp = [write_sparse(str(tmp_path / n), P, 16, rng) for n, P in (("sP1", P1), ("sP2", P2))]
    kw = dict(nk=s.nk, nb_dm=s.nb_dm, bstart=s.bstart, bend=s.bend, e_dm=s.e_dm, k1st=s.k1st, k2nd=s.k2nd,
              prefac_eph=s.prefac_eph, Hcoh=s.Hcoh, picture=s.picture_schrodinger, expt=s.expt, precision=prec,
              f_ref=s.f_dm if prec == "bf16x2" else None)
    y = oracle.y_of(s.dm0)
    t = 31.0 * oracle.fs
    with LindbladGPU(P1=P1.reshape(-1), P2=P2.reshape(-1), **kw) as gd:
        rd = gd.func(t, y)
    with LindbladGPU(P1=None, P2=None, P_sparse=sp, **kw) as gs:
        rs = gs.func(t, y)
    assert rel(rs, rd) <= (1e-15 if prec == "f64x" else 1e-12)


@pytest.mark.parametrize("prec", ["f64", "f64x"])
def test_t2_in_transverse_field_from_gpu_trajectory(prec, oracle, built):
    """T2: S_z precessing about the 2 T in-plane field of nb2_eimp_B (initial spin along z), fitted
    with the decaying-cosine model of fit.py (the field sets omega); S(t) within 1e-10 of the oracle's,
    and the lifetime and precession period of the least-squares optimum converged to machine
    precision within 1e-10 (the fit.py-faithful leastsq values stop at its xtol, ~1e-8)."""
    from denmat_dynm_development_gb300.t1fit import fit_t1
    s = oracle.load(os.path.join(GOLDEN, "nb2_eimp_B"))
    h, nsteps, every = 10.0 * oracle.fs, 3000, 50
    y0 = oracle.y_of(s.dm0)
    _, rec_o = oracle.rk4(s, s.t0, h, nsteps, y0, every=every)
    with make_gpu(s, prec) as gpu:
        gpu.set_state(s.t0, y0)
        gpu.set_observable(0, s.smat[:, 2, :], s.f_dm, s.ob_prefac)
        rec = []
        for _ in range(nsteps // every):
            gpu.rk4(h, every)
            t, _ = gpu.get_state()
            rec.append((t,) + gpu.measure(0, s.nv_dm))
    rec = np.array(rec)
    assert rel(rec[:, 1], rec_o[:, 1]) < 1e-10
    fo = fit_t1(rec_o[:, 0], rec_o[:, 1], bfield_tesla=2.0)
    fg = fit_t1(rec[:, 0], rec[:, 1], bfield_tesla=2.0)
    err = abs(fg.tau_conv - fo.tau_conv) / abs(fo.tau_conv)
    errp = abs(fg.period_conv - fo.period_conv) / abs(fo.period_conv)
    print("%s: T2 oracle %.15g ps gpu %.15g ps (converged fit), rel err %.3g, period rel err %.3g"
          % (prec, fo.tau_conv, fg.tau_conv, err, errp))
    assert np.isfinite(fo.tau_conv) and np.isfinite(fg.tau_conv)
    assert err < 1e-10 and errp < 1e-10
    assert abs(fg.tau_lsq - fo.tau_lsq) / abs(fo.tau_lsq) < 1e-6


def test_bounded_wait_gives_up_and_reports_a_timeout(oracle, built):
    """A bulk-copy wait that cannot complete (an mbarrier phase nothing completes) gives up after its
    poll limit and raises the device flag: the host reads DMD_E_TIMEOUT, the context stays usable
    (the self-test runs a kernel afterwards, and a handle steps normally after it)."""
    import ctypes as C
    from denmat_dynm_development_gb300 import dmd
    L = dmd._lib()
    st = C.c_int(-1)
    assert L.dmd_selftest_wait_timeout(0, 256, C.byref(st)) == 0
    assert st.value == 5  # DMD_E_TIMEOUT
    s = oracle.load(os.path.join(GOLDEN, "nb2_eimp_B"))
    with make_gpu(s, "f64x") as gpu:
        gpu.set_state(s.t0, oracle.y_of(s.dm0))
        gpu.rk4(1.0 * oracle.fs, 3)
        _, y = gpu.get_state()
        assert np.all(np.isfinite(y))


def _random_system(oracle, nk, nb_dm, bstart, bend, npair, seed, with_H=True, picture=0):
    """a random system with an arbitrary band window: random Hermitian states, energies, operators
    (the RHS needs no structure of P) and pairs drawn with repeats and either orientation"""
    rng = np.random.default_rng(seed)
    nb = bend - bstart
    e = np.sort(rng.uniform(0.05, 0.06, (nk, nb_dm)), axis=1)
    f = 1.0 / (np.exp((e - 0.052) / 9.5e-4) + 1.0)
    k1 = rng.integers(0, nk, npair).astype(np.uint64)
    k2 = rng.integers(0, nk, npair).astype(np.uint64)
    P1 = (rng.standard_normal((npair, nb ** 4)) + 1j * rng.standard_normal((npair, nb ** 4))) * 1e-3
    P2 = (rng.standard_normal((npair, nb ** 4)) + 1j * rng.standard_normal((npair, nb ** 4))) * 1e-3
    dm = rng.standard_normal((nk, nb_dm, nb_dm)) + 1j * rng.standard_normal((nk, nb_dm, nb_dm))
    dm = 1e-3 * 0.5 * (dm + np.conj(np.swapaxes(dm, 1, 2)))
    dm[:, range(nb_dm), range(nb_dm)] = f + 1e-3 * rng.standard_normal((nk, nb_dm))
    H = None
    if with_H:
        H = rng.standard_normal((nk, nb_dm, nb_dm)) + 1j * rng.standard_normal((nk, nb_dm, nb_dm))
        H = 1e-6 * 0.5 * (H + np.conj(np.swapaxes(H, 1, 2)))
        if picture == 1:  # the Schrodinger picture's H carries the band energies
            H[:, range(nb_dm), range(nb_dm)] += e
        H = H.reshape(nk, -1)
    return oracle.from_arrays(nk=nk, nb_dm=nb_dm, bstart=bstart, bend=bend, e_dm=e, f_dm=f, k1st=k1, k2nd=k2,
                              P1=P1.reshape(-1), P2=P2.reshape(-1), prefac_eph=2 * np.pi / 1e5,
                              dm0=dm.reshape(nk, -1), Hcoh=H, picture_schrodinger=picture, expt=1 - picture,
                              smat=np.zeros((nk, 3, nb_dm * nb_dm), np.complex128))


@pytest.mark.parametrize("nb_dm,bstart,bend,npair,picture", [(3, 0, 3, 150, 0), (1, 0, 1, 80, 1), (4, 1, 4, 60, 0),
                                                             (2, 0, 2, 0, 0), (3, 1, 2, 50, 1)])
def test_band_windows_and_empty_pairs_vs_oracle(nb_dm, bstart, bend, npair, picture, oracle, built):
    """Windows outside the column-block form (nb = 1, 3 on the per-thread FP64 kernel, including a
    window inside the density matrix), a system without k-pairs (the coherent term alone), both
    pictures: the FP64 RHS and 5 RK4 steps against the oracle."""
    s = _random_system(oracle, 23, nb_dm, bstart, bend, npair, seed=nb_dm * 10 + npair, picture=picture)
    y = oracle.y_of(s.dm0)
    t = 5.0 * oracle.fs
    with make_gpu(s, "f64") as gpu:
        e = rel(gpu.func(t, y), oracle.rhs(s, t, y))
        gpu.set_state(0.0, y)
        gpu.rk4(1.0 * oracle.fs, 5)
        _, yg = gpu.get_state()
    yo, _ = oracle.rk4(s, 0.0, 1.0 * oracle.fs, 5, y)
    e2 = rel(yg - y, yo - y)
    print("nb_dm %d window [%d,%d) npair %d picture %d: RHS rel err %.3g, 5-step change %.3g"
          % (nb_dm, bstart, bend, npair, picture, e, e2))
    assert e < RHS_TOL["f64"] and e2 < 1e-11
