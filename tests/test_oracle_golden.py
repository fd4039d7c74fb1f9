"""Pin the oracle: the CPU restatement against vectors produced by the reference's own sources.

tests/golden/<case>/golden.npz was written by tests/golden/make_golden.py from the shim-built
reference program (DMD src_v4.5.7 compiled unmodified). The restatement shares the reference
build's BLAS definitions and C library, so set-up and right-hand side must agree bit for bit;
the steppers must agree to rounding of the printed S(t) files.
"""
import os

import numpy as np
import pytest

from conftest import EE_CASES, GOLDEN, GOLDEN_CASES


def _load(case, oracle):
    d = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(d, "golden.npz")))
    s = oracle.load(d)
    return d, g, s


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_setup_bitwise(case, oracle):
    d, g, s = _load(case, oracle)
    meta = dict(zip(g["meta_keys"], g["meta_vals"]))
    assert s.nk == int(meta["nk"]) and s.nb_dm == int(meta["nb_dm"])
    assert s.bstart == int(meta["bstart"]) and s.bend == int(meta["bend"])
    assert s.npair == int(meta["nkpair"])
    assert s.prefac_eph == meta["prefac_eph"]
    np.testing.assert_array_equal(s.e_dm, g["e_dm"])
    np.testing.assert_array_equal(s.f_dm, g["f_dm"])
    np.testing.assert_array_equal(s.dm0, g["dm0"])
    if "Hcoh" in g:
        np.testing.assert_array_equal(s.Hcoh, g["Hcoh"])
    else:
        assert s.Hcoh is None
    assert s.mu == meta["mu"]
    assert s.nv_dm == int(meta["nv_dm"])
    if meta["ddmdteq"]:
        # set_dm_eq (chemical potentials keeping the carrier numbers) and compute_ddmdt_eq
        assert s.mue == meta["mue"] and s.muh == meta["muh"]
        np.testing.assert_array_equal(s.f_eq, g["f_eq"])
        np.testing.assert_array_equal(s.ddmdt_eq, g["ddmdt_eq"])
    else:
        assert s.ddmdt_eq is None
    if meta["linearize"]:
        # set_dm_eq and set_Lsc (the linear operators replace P1, P2)
        assert s.mue == meta["mue"] and s.muh == meta["muh"]
        np.testing.assert_array_equal(s.f_eq, g["f_eq"])
        np.testing.assert_array_equal(s.P1.reshape(g["Lscij"].shape), g["Lscij"])
        np.testing.assert_array_equal(s.P2.reshape(g["Lscji"].shape), g["Lscji"])


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_rhs_bitwise(case, oracle):
    d, g, s = _load(case, oracle)
    for i, t in enumerate(g["rhs_t"]):
        y = g["rhs_y"][i]
        np.testing.assert_array_equal(oracle.rhs(s, t, y), g["rhs_dydt"][i])
        eph, coh = oracle.rhs_parts(s, t, y)
        np.testing.assert_array_equal(eph, g["rhs_eph"][i])
        np.testing.assert_array_equal(coh, g["rhs_coh"][i])


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_rk4_trajectory(case, oracle):
    d, g, s = _load(case, oracle)
    y, rec = oracle.rk4(s, s.t0, 1.0 * oracle.fs, 40, oracle.y_of(s.dm0), every=5, idir=2)
    np.testing.assert_array_equal(y, g["rk4_y"])
    ref = g["rk4_sz"][1:]  # first row is report(0) at t0
    assert rec.shape[0] == ref.shape[0]
    # the S file is printed with %21.14le (15 significant digits)
    np.testing.assert_allclose(rec[:, 0], ref[:, 0], rtol=2e-14)
    np.testing.assert_allclose(rec[:, 1], ref[:, 1], rtol=2e-14, atol=1e-300)
    np.testing.assert_allclose(rec[:, 2], ref[:, 2], rtol=2e-14, atol=1e-300)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_rkf45_gsl_driver(case, oracle):
    d, g, s = _load(case, oracle)
    st, y, rec, ncalls = oracle.rkf45(s, oracle.y_of(s.dm0), s.t0, s.tend, s.tstep, s.ode["hstart"], s.ode["hmin"],
                                      s.ode["hmax"], s.ode["epsabs"])
    assert st == 0
    np.testing.assert_array_equal(y, g["gsl_y"])
    ref = g["gsl_sz"][1:]
    assert rec.shape[0] == ref.shape[0]
    np.testing.assert_allclose(rec[:, 1], ref[:, 1], rtol=2e-14, atol=1e-300)
    # the reference resets ncalls after its first compute() (report_tau at it = 1)
    np.testing.assert_array_equal(ncalls, g["gsl_ncalls"])


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_euler_driver(case, oracle):
    """DMD's own evolve_euler (DensityMatrix_Dynamics.h:176-186, 229-233): steps of tstep while
    t < tend, t advanced by repeated addition (the loop takes a 21st step when 20 sums of 1 fs fall
    short of tend), dm += dt/2 (ddmdt + ddmdt^dagger) (update_dm_euler, DenMat.cpp:236-248); the
    final state bitwise and S_z at every step to the S file's printed digits"""
    d, g, s = _load(case, oracle)
    y = oracle.y_of(s.dm0)
    t = s.t0
    rec = []
    while t < s.tend:
        y = oracle.euler(s, t, s.tstep, 1, y)
        t += s.tstep
        rec.append((t,) + oracle.measure(s, y, t))
    np.testing.assert_array_equal(y, g["euler_y"])
    rec = np.array(rec)
    ref = g["euler_sz"][1:]  # first row is report(0) at t0
    assert rec.shape[0] == ref.shape[0]
    np.testing.assert_allclose(rec[:, 0], ref[:, 0], rtol=2e-14)
    np.testing.assert_allclose(rec[:, 1], ref[:, 1], rtol=2e-14, atol=1e-300)
    np.testing.assert_allclose(rec[:, 2], ref[:, 2], rtol=2e-14, atol=1e-300)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_hermiticity_of_rhs(case, oracle):
    """dρ/dt is exactly Hermitian: (c + c†)/2 in the finish (evolve_eph.cpp:149-151)."""
    d, g, s = _load(case, oracle)
    eph = g["rhs_eph"][0].view(np.complex128).reshape(s.nk, s.nb_dm, s.nb_dm)
    np.testing.assert_array_equal(eph, np.conj(np.swapaxes(eph, 1, 2)))


@pytest.mark.parametrize("nproc", [1, 3])
def test_rank_sliced_rhs_matches(nproc, oracle):
    """The multi-process CPU baseline (DMD's MPI decomposition) equals the single-rank RHS up to the
    order of the allreduce sum."""
    d = os.path.join(GOLDEN, "nb2_eimp_B")
    s = oracle.load(d)
    y = oracle.y_of(s.dm0)
    t = 17.0 * oracle.fs
    ref = oracle.rhs(s, t, y)
    par = oracle.ParallelRHS(s, nproc)
    try:
        out = par(t, y)
    finally:
        par.close()
    assert np.abs(out - ref).max() <= 1e-14 * np.abs(ref).max()
    if nproc == 1:
        np.testing.assert_array_equal(out, ref)


@pytest.mark.parametrize("case", EE_CASES)
def test_ee_operators_bitwise(case, oracle):
    """e-e model (eeMode = Pee_update): the operators after set-up (P_ee at the equilibrium
    occupations) and after reset_scatt on three states (screening density from each state, P_ee(rho))
    equal the reference's bit for bit."""
    d = os.path.join(GOLDEN, case)
    g = np.load(os.path.join(d, "golden.npz"))
    s = oracle.load(d)
    nb4 = (s.bend - s.bstart) ** 4
    np.testing.assert_array_equal(s.P1.reshape(-1, nb4), g["ee_P1_eq"])
    np.testing.assert_array_equal(s.P2.reshape(-1, nb4), g["ee_P2_eq"])
    for i, (t, y) in enumerate(zip(g["rhs_t"], g["rhs_y"])):
        P1, P2 = oracle.ee_rebuild(s, t, y)
        np.testing.assert_array_equal(P1.reshape(-1, nb4), g["pee_P1"][i])
        np.testing.assert_array_equal(P2.reshape(-1, nb4), g["pee_P2"][i])
        assert s.ee.nfree == g["pee_nfree"][i]


def test_ee_cases_cover_the_model():
    """the e-e golden cases span the screening formulas, the exchange term, both pictures and nb = 2, 4"""
    seen = set()
    for case in EE_CASES:
        from oracle.oracle import parse_param_in
        pm = parse_param_in(os.path.join(GOLDEN, case, "param.in"))
        seen.add(pm["scrFormula"])
        seen.add("anti" if pm.get("ee_antisymmetry", "0") == "1" else "direct")
        seen.add(pm.get("alg_picture", "interaction"))
    assert {"debye", "Bechstedt", "unscreened", "RPA", "anti", "direct", "schrodinger", "interaction"} <= seen
