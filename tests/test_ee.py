"""e-e operators rebuilt from the density matrix (eeMode = Pee_update) on the GPU.

The golden cases (tests/golden/ee_*) come from the reference's own code: the operators after set-up
and after reset_scatt on three states, the RHS with the rebuild before every evaluation (func), 40
RK4 steps through it and the S_z record. The GPU path is checked against them and against the FP64
oracle (oracle/dmd_oracle.c: orc_ee_P, orc_ee_rebuild), which equals the reference bit for bit on
these cases (tests/test_oracle_golden.py). Tolerances: 1e-12 relative for the FP64 operators (the
GPU sums in another order and with FMA), the RHS tolerances of the plain paths, 1e-10 for the
trajectories.
"""
import os

import numpy as np
import pytest

from conftest import EE_CASES, FIXED_P_CASES, GOLDEN

pytestmark = pytest.mark.gpu

P_TOL = 1e-12
# handles of the FP32-pair arithmetic build P_ee with double-float contractions (~2^-47 per product)
P_TOL_DF = 5e-12
RHS_TOL = {"f64": 1e-12, "f64x": 1e-11, "f32": 2e-6, "bf16x2": 2e-5}


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as G
    G.build()


def ee_desc(s, every_rhs=None):
    e = s.ee
    return dict(kvec=e.kvec, kmesh=e.kmesh, U=e.U, f=np.ascontiguousarray(s.f_dm[:, s.bstart:s.bend]), GGT=e.GGT,
                cell_size=e.cell_size, nk_full=e.nk_full, temperature=e.T, eps_background=e.eps, meff=e.meff,
                formula=e.formula, nfree=e.c.nfree, update_screening=e.update_screening, nv=e.nv,
                degauss=e.degauss, ethr=e.ethr, antisymmetry=e.antisym, scale=e.scale,
                every_rhs=e.inside if every_rhs is None else every_rhs, dynamic=e.dynamic, ppa_gn=e.ppa_gn,
                eppa=e.eppa, smearing=e.smearing, two_freqs=e.two_freqs)


def make_ee_gpu(s, prec="f64", every_rhs=None):
    """a handle over P_base = P_eph (+ P_eimp) with the e-e model attached (set-up: P_ee at f); with
    the equilibrium drift (alg_ddmdteq) P_ee rebuilt at rho_eq = diag(f_eq) as the reference's set-up
    does (DensityMatrix_Dynamics.h:58-63) and the drift installed"""
    from denmat_dynm_development_gb300.dmd import LindbladGPU
    dev = prec in ("f32", "bf16x2")
    g = LindbladGPU(nk=s.nk, nb_dm=s.nb_dm, bstart=s.bstart, bend=s.bend, e_dm=s.e_dm, k1st=s.k1st, k2nd=s.k2nd,
                    P1=s.ee.P1base, P2=s.ee.P2base, prefac_eph=s.prefac_eph, Hcoh=s.Hcoh,
                    picture=s.picture_schrodinger, expt=s.expt, precision=prec,
                    f_ref=s.f_dm if dev else None, ee=ee_desc(s, every_rhs))
    if s.ddmdt_eq is not None:
        dm_eq = np.zeros((s.nk, s.nb_dm, s.nb_dm), np.complex128)
        dm_eq[:, range(s.nb_dm), range(s.nb_dm)] = s.f_eq
        g.set_state(0.0, np.ascontiguousarray(dm_eq.reshape(s.nk, -1)).view(np.float64).reshape(-1).copy())
        g.ee_update()
        g.set_ddmdt_eq(s.ddmdt_eq)
    return g


def fresh(oracle, case):
    d = os.path.join(GOLDEN, case)
    return oracle.load(d), dict(np.load(os.path.join(d, "golden.npz")))


@pytest.mark.parametrize("prec", ["f64", "f64x"])
@pytest.mark.parametrize("case", EE_CASES)
def test_ee_setup_and_rebuilds_vs_golden(case, prec, oracle, built):
    """P_ee at set-up (equilibrium occupations, set-up screening) and after dmd_ee_update on the three
    golden states: P_base + scale P_ee and the screening density match the reference's (FP64
    contractions for f64 handles, double-float for f64x)."""
    s, g = fresh(oracle, case)
    nb4 = (s.bend - s.bstart) ** 4
    tol = P_TOL if prec == "f64" else P_TOL_DF
    B1, B2 = s.ee.P1base.reshape(-1, nb4), s.ee.P2base.reshape(-1, nb4)
    with make_ee_gpu(s, prec, every_rhs=0) as gpu:
        P1, P2, n0 = gpu.ee_read()
        e1 = rel(B1 + s.ee.scale * P1, g["ee_P1_eq"])
        e2 = rel(B2 + s.ee.scale * P2, g["ee_P2_eq"])
        print("%s %s set-up: P rel err %.3g %.3g" % (case, prec, e1, e2))
        assert e1 < tol and e2 < tol
        if s.ddmdt_eq is None:  # the set-up density itself
            assert n0 == s.ee.c.nfree
        else:  # the density of rho_eq, summed on the device
            assert abs(n0 - s.ee.c.nfree) <= 1e-14 * abs(s.ee.c.nfree)
        for i, (t, y) in enumerate(zip(g["rhs_t"], g["rhs_y"])):
            gpu.set_state(t, y)
            gpu.ee_update()
            P1, P2, n = gpu.ee_read()
            e1 = rel(B1 + s.ee.scale * P1, g["pee_P1"][i].reshape(-1, nb4))
            e2 = rel(B2 + s.ee.scale * P2, g["pee_P2"][i].reshape(-1, nb4))
            print("%s %s state %d: P rel err %.3g %.3g, nfree %.17g vs %.17g" % (case, prec, i, e1, e2, n,
                                                                                 g["pee_nfree"][i]))
            assert e1 < tol and e2 < tol
            assert abs(n - g["pee_nfree"][i]) <= 1e-14 * abs(g["pee_nfree"][i])


@pytest.mark.parametrize("prec", ["f64", "f64x"])
@pytest.mark.parametrize("case", EE_CASES)
def test_ee_rhs_with_rebuild_vs_golden(case, prec, oracle, built):
    """dmd_func with the rebuild before every evaluation (freq_update_ee_model < 0) equals the
    reference's func on the golden states, at any order of calls."""
    s, g = fresh(oracle, case)
    with make_ee_gpu(s, prec) as gpu:
        for i in (2, 0, 1, 2):
            e = rel(gpu.func(g["rhs_t"][i], g["rhs_y"][i]), g["rhs_dydt"][i])
            print("%s %s state %d: rel err %.3g" % (case, prec, i, e))
            assert e < RHS_TOL[prec]


@pytest.mark.parametrize("prec", ["f64", "f64x"])
@pytest.mark.parametrize("case", EE_CASES)
def test_ee_rk4_trajectory_vs_golden(case, prec, oracle, built):
    """40 RK4 steps of 1 fs in captured graphs, every stage rebuilding P_ee on the device: the final
    state and S_z every 5 steps match the reference's."""
    s, g = fresh(oracle, case)
    fs = oracle.fs
    with make_ee_gpu(s, prec) as gpu:
        gpu.set_state(s.t0, oracle.y_of(s.dm0))
        gpu.set_observable(0, s.smat[:, 2, :], s.f_dm, s.ob_prefac)
        sz = []
        for _ in range(8):
            gpu.rk4(1.0 * fs, 5)
            sz.append(gpu.measure(0, s.nv_dm)[0])
        _, y = gpu.get_state()
    ey = rel(y - oracle.y_of(s.dm0), g["rk4_y"] - oracle.y_of(s.dm0))
    es = rel(sz, g["rk4_sz"][1:, 1])
    print("%s %s: 40-step change rel err %.3g, S_z rel err %.3g" % (case, prec, ey, es))
    assert ey < 1e-10 and es < 1e-10


@pytest.mark.parametrize("case", ["ee_nb2_debye", "ee_nb4_unscreened"])
def test_ee_updates_between_steps_vs_oracle(case, oracle, built):
    """freq_update_ee_model > 0: P_ee rebuilt from the state every 4 steps (dmd_ee_update between
    dmd_rk4 calls, update_scatt_outside) against the oracle doing the same."""
    s, g = fresh(oracle, case)
    h = 2.0 * oracle.fs
    s.ee.c.inside = 0  # the oracle rebuilds only where the test says
    y = oracle.y_of(s.dm0)
    t = s.t0
    with make_ee_gpu(s, every_rhs=0) as gpu:
        gpu.set_state(t, y)
        for blk in range(5):
            gpu.ee_update()
            gpu.rk4(h, 4)
            oracle.ee_rebuild(s, t, y)
            y, _ = oracle.rk4(s, t, h, 4, y)
            t = t + 4 * h
            _, yg = gpu.get_state()
            e = rel(yg - oracle.y_of(s.dm0), y - oracle.y_of(s.dm0))
            print("%s block %d: change rel err %.3g" % (case, blk, e))
            assert e < 1e-10


@pytest.mark.parametrize("prec", ["f32", "bf16x2"])
def test_ee_reduced_precision_rhs(prec, oracle, built):
    """the deviation forms refill their constant term with the operators: RHS with the rebuild at
    their reduced-precision tolerance"""
    s, g = fresh(oracle, "ee_nb2_debye")
    with make_ee_gpu(s, prec) as gpu:
        for i in range(3):
            e = rel(gpu.func(g["rhs_t"][i], g["rhs_y"][i]), g["rhs_dydt"][i])
            print("ee_nb2_debye %s state %d: rel err %.3g" % (prec, i, e))
            assert e < RHS_TOL[prec]


@pytest.mark.parametrize("prec", ["f64", "f64x"])
def test_ee_larger_random_case_vs_oracle(prec, oracle, built, tmp_path):
    """a denser ball of k-points (nk = 120, ~6k pairs, many k3 per pair) with the exchange term:
    P_ee from a perturbed state against the oracle"""
    from denmat_dynm_development_gb300.ldbd_synth import SynthConfig, make_ldbd
    cfg = SynthConfig(nk=120, nb=2, seed=41, de_pair_mev=60.0, nwannier=4, kball=True)
    extra = {"eeMode": "Pee_update", "scrMode": "medium", "freq_update_ee_model": -1, "freq_update_eimp_model": -1,
             "epsilon_background": 12.9, "scrFormula": "debye", "update_screening": 1, "ee_antisymmetry": 1}
    make_ldbd(str(tmp_path), cfg, B_T=(0.4, 0, 0), extra=extra)
    s = oracle.load(str(tmp_path))
    rng = np.random.default_rng(5)
    dm = s.dm0.reshape(s.nk, s.nb_dm, s.nb_dm) + 2e-4 * (rng.standard_normal((s.nk, s.nb_dm, s.nb_dm)) +
                                                        1j * rng.standard_normal((s.nk, s.nb_dm, s.nb_dm)))
    dm = 0.5 * (dm + np.conj(np.swapaxes(dm, 1, 2)))
    y = oracle.y_of(dm.reshape(s.nk, -1))
    t = 13.0 * oracle.fs
    with make_ee_gpu(s, prec, every_rhs=0) as gpu:
        gpu.set_state(t, y)
        gpu.ee_update()
        P1, P2, n = gpu.ee_read()
    oracle.ee_rebuild(s, t, y)
    e1, e2 = rel(P1, s.ee.P1ee.reshape(P1.shape)), rel(P2, s.ee.P2ee.reshape(P2.shape))
    print("nk120 %s npair %d: P_ee rel err %.3g %.3g, nfree %.17g vs %.17g" % (prec, s.npair, e1, e2, n, s.ee.nfree))
    tol = P_TOL if prec == "f64" else P_TOL_DF
    assert e1 < tol and e2 < tol
    assert abs(n - s.ee.nfree) <= 1e-14 * abs(s.ee.nfree)


@pytest.mark.parametrize("case", EE_CASES)
def test_ee_host_library_rkf45_vs_golden_gsl(case, oracle, built):
    """The host library path (dmdh_load of param.in with eeMode = Pee_update, dmdh_prepare attaching
    the model) through DMD's evolve_gsl loop: S_z per output interval, the final state and the RHS
    calls per interval equal the reference's evolve_gsl with the rebuild before every evaluation."""
    from denmat_dynm_development_gb300 import host
    d = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(d, "golden.npz")))
    s = oracle.load(d)
    hs_sys = host.System(d)
    with hs_sys.gpu("f64") as gpu:
        gpu.set_state(s.t0, oracle.y_of(s.dm0))
        gpu.set_observable(0, s.smat[:, 2, :], s.f_dm, s.ob_prefac)
        hs, ti, tcur = s.ode["hstart"], s.t0, s.t0
        sz, nf = [], []
        while tcur < s.tend:
            ti += s.tstep
            hs, n = gpu.rkf45_apply(ti, hs, s.ode["hmin"], s.ode["hmax"], s.ode["epsabs"], 0.0)
            tcur, _ = gpu.get_state()
            sz.append(gpu.measure(0, s.nv_dm)[0])
            nf.append(n)
        _, y = gpu.get_state()
    hs_sys.close()
    e = rel(np.array(sz), g["gsl_sz"][1:, 1])
    print("%s: RKF45 S_z rel err %.3g, state %.3g, ncalls %s" % (case, e, rel(y, g["gsl_y"]), nf))
    assert rel(y, g["gsl_y"]) < 1e-10 and e < 1e-10
    np.testing.assert_array_equal(np.array(nf), g["gsl_ncalls"])


def test_ee_argument_and_order_checks(oracle, built):
    """dmd_ee_attach needs DMD_FLAG_EE (DMD_E_STATE without it), a second attach is refused, update and
    read need an attached model, the flag is refused with the adjoint and for batches, and a bad
    description is DMD_E_ARG; the handle stays usable after each refusal."""
    from denmat_dynm_development_gb300.dmd import DMDError, LindbladGPU
    s, g = fresh(oracle, "ee_nb2_debye")
    common = dict(nk=s.nk, nb_dm=s.nb_dm, bstart=s.bstart, bend=s.bend, e_dm=s.e_dm, k1st=s.k1st, k2nd=s.k2nd,
                  P1=s.ee.P1base, P2=s.ee.P2base, prefac_eph=s.prefac_eph, Hcoh=s.Hcoh, picture=s.picture_schrodinger,
                  expt=s.expt)
    with LindbladGPU(precision="f64", **common) as plain:
        with pytest.raises(DMDError) as ex:
            plain.ee_attach(**ee_desc(s))
        assert ex.value.status == 7  # DMD_E_STATE
        with pytest.raises(DMDError):
            plain.ee_update()
        out = plain.func(g["rhs_t"][0], g["rhs_y"][0])
        assert np.isfinite(out).all()
    for kw in (dict(adjoint=True), dict(nrhs=2, precision="bf16x2", f_ref=s.f_dm)):
        args = dict(common, precision="f64")
        args.update(kw)
        with pytest.raises(DMDError) as ex:
            LindbladGPU(ee_flag=True, **args)
        assert ex.value.status == 1  # DMD_E_ARG
    with LindbladGPU(precision="f64", ee_flag=True, **common) as gpu:
        bad = ee_desc(s)
        bad["degauss"] = 0.0
        with pytest.raises(DMDError) as ex:
            gpu.ee_attach(**bad)
        assert ex.value.status == 1
        for key, val in (("dynamic", 1), ("two_freqs", 1)):  # ppa needs RPA; two frequencies need ppa
            bad = ee_desc(s)
            bad[key] = val
            with pytest.raises(DMDError) as ex:
                gpu.ee_attach(**bad)
            assert ex.value.status == 1
        gpu.ee_attach(**ee_desc(s))
        with pytest.raises(DMDError) as ex:
            gpu.ee_attach(**ee_desc(s))
        assert ex.value.status == 7
        e = rel(gpu.func(g["rhs_t"][1], g["rhs_y"][1]), g["rhs_dydt"][1])
        assert e < RHS_TOL["f64"]


LINEAR_EE_CASES = [c for c in FIXED_P_CASES if c.startswith("ee_") and "linear" in c]


@pytest.mark.gpu
@pytest.mark.parametrize("case", LINEAR_EE_CASES)
def test_linearized_ee_source_vs_reference(case, oracle, built):
    """The e-e source of the linearized operators (add_Lsc_contrib("ee"): P_ee at f_eq and, unless
    eeMode = Pee_fixed_at_eq, the P3..P6 terms), built by the host library with the GPU
    (dmd_ee_linear_terms): the operators within 1e-12 of the reference's Lscij / Lscji, and the RHS
    and 40 RK4 steps of the resulting linearized system against the reference's."""
    from denmat_dynm_development_gb300.host import System
    d = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(d, "golden.npz")))
    s = System(d)
    e1 = rel(s.P1.reshape(g["Lscij"].shape), g["Lscij"])
    e2 = rel(s.P2.reshape(g["Lscji"].shape), g["Lscji"])
    print("%s: Lscij rel err %.3g, Lscji %.3g" % (case, e1, e2))
    assert e1 < 1e-12 and e2 < 1e-12
    with s.gpu("f64") as gpu:
        for i, t in enumerate(g["rhs_t"]):
            assert rel(gpu.func(t, g["rhs_y"][i]), g["rhs_dydt"][i]) < 1e-12
        gpu.set_state(s.info.t0, np.ascontiguousarray(s.dm0).view(np.float64).reshape(-1))
        gpu.rk4(1.0 * oracle.fs, 40)
        _, y = gpu.get_state()
    assert rel(y, g["rk4_y"]) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["ee_nb2_linear", "ee_nb4_linear_rpa_anti"])
def test_p3_to_p6_on_gpu_vs_oracle(case, oracle, built):
    """dmd_ee_linear_terms' P_ee at f_eq and P3..P6 (k_ee_p36) against the oracle's restatement of
    calc_P / calc_P3P4 / calc_P5P6 on the same inputs, 1e-12 normwise each."""
    from denmat_dynm_development_gb300.dmd import LindbladGPU
    from denmat_dynm_development_gb300.host import System
    d = os.path.join(GOLDEN, case)
    s = System(d)
    o = oracle.load(d)
    ee = s.ee
    assert ee is not None and o.lin_ee is not None
    i = s.info
    nb = i.bend - i.bstart
    f_lin = np.ascontiguousarray(s.f_eq[:, i.bstart:i.bend])
    n = ee["nfree"]
    if ee["update_screening"]:  # coulomb_model::init(f_eq)
        n = float(sum((1 - f_lin[k, b]) if b < ee["nv"] else f_lin[k, b] for k in range(i.nk) for b in range(nb)))
        n /= ee["nk_full"] * ee["cell_size"]
    base = np.zeros(o.npair * nb ** 4, np.complex128)
    with LindbladGPU(nk=o.nk, nb_dm=o.nb_dm, bstart=o.bstart, bend=o.bend, e_dm=o.e_dm, k1st=o.k1st, k2nd=o.k2nd,
                     P1=base, P2=base, prefac_eph=o.prefac_eph, precision="f64", ee=dict(ee, every_rhs=0)) as g:
        got = g.ee_linear_terms(f_lin, n)
    sc = ee["scale"]
    for j, nm in enumerate(["P1ee", "P2ee", "P3", "P4", "P5", "P6"]):
        want = o.lin_ee[j].reshape(o.npair, -1)
        want = want / sc if sc != 1.0 else want
        if np.abs(want).max() == 0:
            assert np.abs(got[j]).max() == 0, nm
            continue
        err = rel(got[j], want)
        print("%s %s rel err %.3g" % (case, nm, err))
        assert err < 1e-12, nm
