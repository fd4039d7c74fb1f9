"""CPU tests of the C++ host library: DMD's readers and set-up against the reference's own outputs
(golden fixtures) and the oracle; file errors and unsupported options fail loudly."""
import os
import shutil

import numpy as np
import pytest

from conftest import EE_CASES, FIXED_P_CASES, GOLDEN, GOLDEN_CASES, ROOT


@pytest.fixture(scope="module")
def host():
    from denmat_dynm_development_gb300 import build as B
    B.build_all()
    from denmat_dynm_development_gb300 import host as H
    return H


def test_host_exports_header(host):
    import ctypes as C
    import re
    src = open(os.path.join(ROOT, "include", "dmd_host.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = sorted(set(re.findall(r"\b(dmdh_[a-z0-9_A-Z]+)\s*\(", src)))
    L = C.CDLL(host.HOST_LIB)
    assert not [n for n in names if not hasattr(L, n)]
    assert sorted(host.EXPORTS) == names


# the linearized e-e cases build their e-e source on the GPU (tests/test_ee.py checks them there)
CPU_SETUP_CASES = [c for c in FIXED_P_CASES if not c.startswith("ee_")]


@pytest.mark.parametrize("case", CPU_SETUP_CASES)
def test_load_matches_reference_setup(case, host, oracle):
    d = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(d, "golden.npz")))
    s = host.System(d)
    meta = dict(zip(g["meta_keys"], g["meta_vals"]))
    assert s.info.nk == int(meta["nk"]) and s.info.nb_dm == int(meta["nb_dm"])
    assert s.info.bstart == int(meta["bstart"]) and s.info.bend == int(meta["bend"])
    assert s.info.nkpair == int(meta["nkpair"])
    assert s.info.prefac_eph == meta["prefac_eph"]
    assert s.info.mu == meta["mu"] and s.info.temperature == meta["temperature"]
    assert s.info.cell_size == meta["cell_size"] and s.info.cell_size_cmd == meta["cell_size_cmd"]
    np.testing.assert_array_equal(s.e_dm, g["e_dm"])
    np.testing.assert_array_equal(s.f_dm, g["f_dm"])
    np.testing.assert_array_equal(s.dm0, g["dm0"])
    if "Hcoh" in g:
        np.testing.assert_array_equal(s.Hcoh, g["Hcoh"])
    else:
        assert s.Hcoh is None
    assert s.info.nv_dm == int(meta["nv_dm"])
    assert s.info.ddmdteq == int(meta["ddmdteq"]) and s.info.linear == int(meta["linearize"])
    if meta["ddmdteq"] or meta["linearize"]:
        assert s.info.mue == meta["mue"] and s.info.muh == meta["muh"]
        np.testing.assert_array_equal(s.f_eq, g["f_eq"])
    else:
        assert s.f_eq is None
    if meta["linearize"]:  # the linear operators replace P1, P2
        np.testing.assert_array_equal(s.P1.reshape(g["Lscij"].shape), g["Lscij"])
        np.testing.assert_array_equal(s.P2.reshape(g["Lscji"].shape), g["Lscji"])
    o = oracle.load(d)
    np.testing.assert_array_equal(s.P1, o.P1)
    np.testing.assert_array_equal(s.P2, o.P2)
    np.testing.assert_array_equal(s.k1st, o.k1st)
    assert s.info.ob_prefac == o.ob_prefac
    assert s.info.tstep == o.tstep and s.info.tend == o.tend
    assert s.info.ode_hstart == o.ode["hstart"] and s.info.ode_hmax == o.ode["hmax"]


def test_truncated_P_file_is_a_file_error(host, tmp_path):
    src = os.path.join(GOLDEN, "nb2_eph")
    dst = str(tmp_path / "case")
    shutil.copytree(src, dst)
    p = os.path.join(dst, "ldbd_data", "ldbd_P1_lindblad.bin")
    with open(p, "r+b") as f:
        f.truncate(os.path.getsize(p) - 16)
    with pytest.raises(RuntimeError, match="size does not match"):
        host.System(dst)


def test_missing_param_and_unsupported_options(host, tmp_path):
    with pytest.raises(RuntimeError, match="param.in does not exist"):
        host.System(str(tmp_path))
    dst = str(tmp_path / "case")
    shutil.copytree(os.path.join(GOLDEN, "nb2_eph"), dst)
    with open(os.path.join(dst, "param.in"), "a") as f:
        f.write("alg_phenom_relax = 1\n")
    with pytest.raises(RuntimeError, match="alg_phenom_relax"):
        host.System(dst)
    dst2 = str(tmp_path / "case2")
    shutil.copytree(os.path.join(GOLDEN, "nb2_eph"), dst2)
    with open(os.path.join(dst2, "param.in"), "a") as f:
        f.write("alg_linearize = 1\nalg_ddmdteq = 1\n")
    with pytest.raises(RuntimeError, match="linearized"):  # parameters.cpp:428-429
        host.System(dst2)


def test_param_parser_quirks(host, tmp_path):
    """map_input drops the character before '=' (parameters.cpp:617): 'key=value' names 'ke'."""
    dst = str(tmp_path / "case")
    shutil.copytree(os.path.join(GOLDEN, "nb2_eph"), dst)
    with open(os.path.join(dst, "param.in"), "a") as f:
        f.write("# comment = 5\nfoo_bar=3\nspam = 1.5 \\\n  2.5\n")
    s = host.System(dst)
    assert s.param("foo_ba") == 3.0
    assert s.param("foo_bar") is None
    assert s.param("spam") == 1.5
    assert s.param("comment") is None


def test_setup_pieces_match_oracle(host, oracle):
    d = os.path.join(GOLDEN, "nb4_eimp_B")
    o = oracle.load(d)
    f = host.fermi(o.temperature, o.mu, o.e_dm)
    np.testing.assert_array_equal(f, o.f_dm)
    Bp = np.array([0.05, 0.0, 0.1]) * oracle.Tesla2au
    dm = host.dm_bpert(o.smat, o.e_dm, o.f_dm, o.temperature, Bp, 0.0, 0)
    np.testing.assert_array_equal(dm, o.dm0)
    # the oracle's own set-up (used where the product library must not be loaded: the benchmark's
    # reference arm) gives the same bits
    np.testing.assert_array_equal(oracle.fermi(o.temperature, o.mu, o.e_dm), f)
    np.testing.assert_array_equal(oracle.dm_bpert(o.smat, o.e_dm, o.f_dm, o.temperature, Bp, 0.0, 0), dm)


@pytest.mark.parametrize("case", EE_CASES)
def test_load_ee_model_matches_reference_setup(case, host, oracle):
    """e-e cases: the host library's e-e descriptor (what dmdh_prepare attaches) equals the reference's
    set-up values (screening density, reciprocal metric, windows) and the oracle's inputs; the base
    operators are P_eph (+ P_eimp) before the e-e term."""
    d = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(d, "golden.npz")))
    meta = dict(zip(g["meta_keys"], g["meta_vals"]))
    s = host.System(d)
    o = oracle.load(d)
    ee = s.ee
    assert ee is not None
    if not meta["ddmdteq"]:
        assert ee["nfree"] == meta["ee_nfree"]
    else:  # the reference's model ends its set-up at rho_eq's density (the reset at rho_eq); the
        # descriptor carries the set-up occupations' density, which attach uses before that reset
        fw = g["f_dm"][:, o.bstart:o.bend]
        nv = ee["nv"]
        n = sum((1 - fw[k, b]) if b < nv else fw[k, b] for k in range(fw.shape[0]) for b in range(fw.shape[1]))
        n /= ee["nk_full"] * ee["cell_size"]
        assert abs(ee["nfree"] - n) <= 1e-13 * abs(n)
        fe = g["f_eq"][:, o.bstart:o.bend]
        n_eq = sum((1 - fe[k, b]) if b < nv else fe[k, b] for k in range(fe.shape[0]) for b in range(fe.shape[1]))
        n_eq /= ee["nk_full"] * ee["cell_size"]
        assert abs(meta["ee_nfree"] - n_eq) <= 1e-13 * abs(n_eq)
    np.testing.assert_array_equal(ee["GGT"], [meta["ee_ggt%d%d" % (i, j)] for i in range(3) for j in range(3)])
    assert ee["degauss"] == meta["ee_degauss"] and ee["ethr"] == meta["ee_ethr"]
    assert ee["eps_background"] == meta["ee_eps"] and ee["meff"] == meta["ee_meff"]
    assert ee["temperature"] == meta["ee_T"] and ee["nv"] == int(meta["ee_nv"])
    assert ee["antisymmetry"] == int(meta["ee_antisym"]) and ee["scale"] == meta["ee_scale"]
    assert ee["every_rhs"] == 1 and ee["formula"] == o.ee.formula and ee["update_screening"] == o.ee.update_screening
    # dynamic screening: the raw parameters (the library applies init_RPA's and :523's defaults)
    assert ee["dynamic"] == o.ee.dynamic and ee["two_freqs"] == o.ee.two_freqs
    if o.ee.dynamic:
        assert ee["ppa_gn"] == o.ee.ppa_gn
        eppa = ee["eppa"] if ee["eppa"] != 0 else np.sqrt(4 * np.pi * ee["nfree"] / ee["meff"] / ee["eps_background"])
        assert eppa == o.ee.eppa
        sm = ee["smearing"] if o.ee.ppa_gn or ee["smearing"] > 0 else 0.5 * ee["temperature"]
        assert sm == o.ee.smearing
    np.testing.assert_array_equal(ee["U"], o.ee.U)
    np.testing.assert_array_equal(ee["kvec"], o.ee.kvec)
    np.testing.assert_array_equal(ee["f"], g["f_dm"][:, o.bstart:o.bend])
    np.testing.assert_array_equal(s.P1, o.ee.P1base.reshape(s.P1.shape))
    np.testing.assert_array_equal(s.P2, o.ee.P2base.reshape(s.P2.shape))
    np.testing.assert_array_equal(s.dm0, g["dm0"])


def test_ee_options_outside_the_path_are_rejected(host, tmp_path):
    for extra, msg in [("scrFormula = heg\n", "scrFormula heg"), ("scrFormula = lindhard\n", "lindhard"),
                       ("dynamic_screening = ppa\n", "static limit"),
                       ("dynamic_screening = real-axis\n", "real-axis"),
                       ("dynamic_screening_ee_two_freqs = 1\n", "only for dynamic screening"),
                       ("alg_linearize_dPee = 1\n", "alg_linearize_dPee"),
                       ("freq_update_eimp_model = 3\n", "freq_update_eimp_model")]:
        dst = str(tmp_path / ("c%d" % len(msg)))
        shutil.copytree(os.path.join(GOLDEN, "ee_nb2_debye"), dst)
        with open(os.path.join(dst, "param.in"), "a") as f:
            f.write(extra)
        with pytest.raises(RuntimeError, match=msg):
            host.System(dst)


def test_rk4_func_validates_its_arguments(host):
    """dmdh_rk4_func refuses a null handle, state or work array before any device call"""
    import ctypes as C
    L = C.CDLL(host.HOST_LIB)
    L.dmdh_rk4_func.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int64, C.c_void_p, C.c_size_t, C.c_void_p]
    y = np.zeros(8)
    w = np.zeros(40)
    assert L.dmdh_rk4_func(None, 0.0, 1.0, 1, y.ctypes.data, y.size, w.ctypes.data) == 1  # DMD_E_ARG
    assert L.dmdh_rk4_func(C.c_void_p(1), 0.0, 1.0, 1, None, y.size, w.ctypes.data) == 1
    assert L.dmdh_rk4_func(C.c_void_p(1), 0.0, 1.0, 1, y.ctypes.data, y.size, None) == 1
    assert L.dmdh_rk4_func(C.c_void_p(1), 0.0, 1.0, -1, y.ctypes.data, y.size, w.ctypes.data) == 1


# the linearized e-e cases load through a GPU handle (their e-e source is built there)
TAU_CPU_CASES = [c for c in GOLDEN_CASES if not (c.startswith("ee_") and "linear" in c)]


@pytest.mark.parametrize("case", TAU_CPU_CASES)
def test_report_tau_writes_the_reference_files(case, host, oracle, tmp_path):
    """dmdh_report_tau at t0 on the set-up state, with dydt the oracle's right-hand side there (the
    oracle equals DMD's func bit for bit), writes the tau files that DMD's evolve_gsl writes at its
    first step (compute + report_tau), byte for byte: the spin directions Bpert selects, electron and
    hole ranges, both pictures' line formats"""
    d = os.path.join(GOLDEN, case)
    g = np.load(os.path.join(d, "golden.npz"))
    s = host.System(d)
    try:
        so = oracle.load(d)
        y0 = s.y0()
        s.report_tau(str(tmp_path), so.t0, y0, oracle.rhs(so, so.t0, y0))
    finally:
        s.close()
    names = sorted(f for f in os.listdir(str(tmp_path)) if f.startswith("tau_"))
    assert names == [str(n) for n in g["gsl_tau_names"]]
    for n, text in zip(names, g["gsl_tau_text"]):
        with open(os.path.join(str(tmp_path), n)) as f:
            assert f.read() == str(text), n


def test_tau_of_a_pure_decay():
    """tau of an observable whose deviation decays as dS/dt = -S/T1 is T1 (without precession)"""
    from denmat_dynm_development_gb300 import host as H
    rng = np.random.default_rng(4)
    nk, nb = 5, 2
    e = np.sort(rng.uniform(0, 0.01, (nk, nb)), axis=1)
    f = rng.uniform(0.1, 0.9, (nk, nb))
    obs = rng.standard_normal((nk, nb, nb)) + 1j * rng.standard_normal((nk, nb, nb))
    obs = 0.5 * (obs + np.conj(np.swapaxes(obs, 1, 2)))
    dev = 1e-3 * (rng.standard_normal((nk, nb, nb)) + 1j * rng.standard_normal((nk, nb, nb)))
    dev = 0.5 * (dev + np.conj(np.swapaxes(dev, 1, 2)))
    dm = dev.copy()
    dm[:, range(nb), range(nb)] += f
    T1 = 1234.5
    tau = H.tau(obs.reshape(nk, -1), e, f, dm.reshape(nk, -1), (-dev / T1).reshape(nk, -1), 0.0, 0.0, picture=1)
    assert tau[0] == 0.0
    assert abs(tau[1] - T1) <= 1e-12 * T1 and abs(tau[2] - T1) <= 1e-12 * T1


@pytest.mark.parametrize("case", ["nb2_eimp_B", "nb2_carrier_eq", "nb2_holes_eq"])
def test_restart_setup_bitwise(case, host, oracle, tmp_path):
    """restart = 1 (parameters.cpp:298-309, read_dm_restart DenMat.cpp:301-316): the state and the
    time read from the restart files the reference's evolve_gsl wrote, and with alg_ddmdteq
    set_dm_eq on that state (chemical potentials, f_eq), equal the reference's restart set-up bit
    for bit; the equilibrium drift from that f_eq (compute_ddmdt_eq at t = 0, evolve_eph.cpp:3-19)
    too, and the tau files of compute + report_tau at the restart time (t0 != 0) byte for byte"""
    import ctypes as C
    import dataclasses
    src = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(src, "golden.npz")))
    d = tmp_path / case
    shutil.copytree(os.path.join(src, "ldbd_data"), str(d / "ldbd_data"))
    with open(os.path.join(src, "param.in")) as f:
        text = f.read()
    assert "restart = 0\n" in text
    (d / "param.in").write_text(text.replace("restart = 0\n", "restart = 1\n"))
    os.makedirs(str(d / "restart"))
    g["restart_in_y"].tofile(str(d / "restart" / "denmat_restart.bin"))
    (d / "restart" / "time_restart.dat").write_text(str(g["restart_in_time"]))
    s = host.System(str(d))
    try:
        np.testing.assert_array_equal(s.dm0, g["restart_dm0"])
        assert s.info.t0 == g["restart_t0"]
        assert s.info.mue == g["restart_mu"][0] and s.info.muh == g["restart_mu"][1]
        if "restart_f_eq" in g:
            np.testing.assert_array_equal(s.f_eq, g["restart_f_eq"])
            so = oracle.load(src)
            drift = np.zeros_like(g["restart_ddmdt_eq"])
            cs = dataclasses.replace(so, Hcoh=None, ddmdt_eq=None).cstruct()
            f_eq = np.ascontiguousarray(s.f_eq)
            oracle.lib().orc_compute_ddmdt_eq(C.addressof(cs), f_eq.ctypes.data, drift.ctypes.data)
            np.testing.assert_array_equal(drift, g["restart_ddmdt_eq"])
        # report_tau at the restart time (t0 != 0) on the restart state, the right-hand side from the
        # oracle with the restart drift: the reference's tau files byte for byte
        so = oracle.load(src)
        if "restart_ddmdt_eq" in g:
            so = dataclasses.replace(so, ddmdt_eq=np.ascontiguousarray(g["restart_ddmdt_eq"]))
        y0 = s.y0()
        out = tmp_path / "tau"
        os.makedirs(str(out))
        s.report_tau(str(out), s.info.t0, y0, oracle.rhs(so, s.info.t0, y0))
        names = sorted(f for f in os.listdir(str(out)) if f.startswith("tau_"))
        assert names == [str(n) for n in g["restart_tau_names"]]
        for n, text in zip(names, g["restart_tau_text"]):
            with open(os.path.join(str(out), n)) as f:
                assert f.read() == str(text), n
    finally:
        s.close()


def test_run_refuses_to_overwrite_an_earlier_run(host, tmp_path):
    """restart = 0 with a restart/ directory present is an error before any device work, as in the
    reference (parameters.cpp:67-68)"""
    src = os.path.join(GOLDEN, "nb2_eimp_B")
    d = tmp_path / "run"
    shutil.copytree(os.path.join(src, "ldbd_data"), str(d / "ldbd_data"))
    shutil.copy(os.path.join(src, "param.in"), str(d))
    os.makedirs(str(d / "restart"))
    with pytest.raises(RuntimeError, match="you should run a restart calculation"):
        host.run(str(d))


@pytest.mark.parametrize("what,match", [
    ("size_short", "ldbd_size.dat is too short"),
    ("size_bands", "inconsistent band ranges"),
    ("size_nk", "ldbd_size.dat line 3"),
    ("no_R", "ldbd_R.dat does not exist"),
    ("ek_truncated", "ldbd_ek.bin"),
    ("no_kpair", "ldbd_kpair_k1st.bin"),
])
def test_broken_inputs_are_file_errors(what, match, host, tmp_path):
    """Host-side fault injection on DMD's inputs (the reference aborts in check_file_size or reads
    garbage): each broken file is a DMD_E_FILE / DMD_E_ARG status with a message, never a crash"""
    dst = str(tmp_path / "case")
    shutil.copytree(os.path.join(GOLDEN, "nb2_eph"), dst)
    ld = os.path.join(dst, "ldbd_data")
    size = os.path.join(ld, "ldbd_size.dat")
    with open(size) as f:
        lines = f.readlines()
    if what == "size_short":
        lines = lines[:5]
    elif what == "size_bands":  # bTop_dm beyond nb
        v = lines[1].split("#")[0].split()
        v[3] = "7"
        lines[1] = " ".join(v) + " # nb nv ...\n"
    elif what == "size_nk":
        lines[2] = "nonsense # nk_full nk kmesh\n"
    elif what == "no_R":
        os.remove(os.path.join(ld, "ldbd_R.dat"))
    elif what == "ek_truncated":
        p = os.path.join(ld, "ldbd_ek.bin")
        with open(p, "r+b") as f:
            f.truncate(os.path.getsize(p) // 2)
    elif what == "no_kpair":
        os.remove(os.path.join(ld, "ldbd_kpair_k1st.bin"))
    with open(size, "w") as f:
        f.writelines(lines)
    with pytest.raises(RuntimeError, match=match):
        host.System(dst)


def test_tau_argument_checks(host):
    """dmdh_tau refuses empty or out-of-range band ranges before reading any array"""
    import ctypes as C
    L = C.CDLL(host.HOST_LIB)
    L.dmdh_tau.argtypes = [C.c_int32, C.c_int32] + [C.c_void_p] * 5 + [C.c_double, C.c_double] + [C.c_int32] * 3 + \
        [C.c_double, C.c_void_p]
    buf = (C.c_double * 64)()
    out = (C.c_double * 3)()
    for nk, nb, b0, b1 in ((1, 2, 1, 1), (1, 2, 0, 3), (1, 2, -1, 1), (0, 2, 0, 2), (1, 0, 0, 0)):
        assert L.dmdh_tau(nk, nb, buf, buf, buf, buf, buf, 0.0, 0.0, 0, b0, b1, 1.0, out) == 1
    assert L.dmdh_tau(1, 2, None, buf, buf, buf, buf, 0.0, 0.0, 0, 0, 2, 1.0, out) == 1
