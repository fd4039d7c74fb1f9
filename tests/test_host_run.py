"""DMD's whole time loop through the host library (dmdh_run) against the reference's own run.

dmdh_run reads param.in and ldbd_data/ from a directory, sets the system up, and runs DMD's
evolve_gsl loop on the GPU, writing DMD's output files there. The golden fixtures hold what the
reference program wrote for the same directory: the S_z file of evolve_gsl (20 output intervals),
its final state (restart/denmat_restart.bin), the tau files of its report_tau at t0, and the RHS
calls per interval. Tolerances: S(t) and the state 1e-10 (the FP64 bound), the tau files to the
printed digits (%14.7le), the RHS-call counts exactly.
"""
import os
import re
import shutil

import numpy as np
import pytest

from conftest import GOLDEN

RUN_CASES = ["nb2_eimp_B", "nb2_holes_eq", "nb2_schrod", "nb4_eimp_B", "ee_nb2_debye"]


def read_s_file(path):
    rows = []
    with open(path) as f:
        for line in f:
            if line.startswith("#") or not line.strip():
                continue
            rows.append([float(x) for x in line.split()])
    return np.array(rows)


def tau_numbers(text):
    """the numbers of a tau file's lines ('<t> fs: <tau> ... ps')"""
    out = []
    for line in text.splitlines():
        if line.startswith("#") or not line.strip():
            continue
        out.append([float(x) for x in line.replace("fs:", " ").replace("ps", " ").split()])
    return np.array(out)


def check_run_dir(rundir, g, stdout, loop="gsl"):
    """compare a run directory (and the run's standard output) with a case's golden records of
    DMD's evolve_gsl (loop = "gsl") or evolve_euler (loop = "euler")"""
    def rel(a, b):
        return float(np.abs(a - b).max() / np.abs(b).max())
    sz = read_s_file(os.path.join(rundir, "sz_elec_tot.out"))
    ref = g[loop + "_sz"]
    assert sz.shape == ref.shape, (sz.shape, ref.shape)
    np.testing.assert_allclose(sz[:, 0], ref[:, 0], rtol=1e-13)
    assert rel(sz[:, 1], ref[:, 1]) < 1e-10 and rel(sz[:, 2], ref[:, 2]) < 1e-10
    y = np.fromfile(os.path.join(rundir, "restart", "denmat_restart.bin"))
    assert rel(y, g[loop + "_y"]) < 1e-10
    names = sorted(f for f in os.listdir(rundir) if f.startswith("tau_") and f.endswith("_tot.out"))
    assert names == [str(n) for n in g["gsl_tau_names"]]
    for n, text in zip(names, g["gsl_tau_text"]):
        with open(os.path.join(rundir, n)) as f:
            got = tau_numbers(f.read())
        np.testing.assert_allclose(got, tau_numbers(str(text)), rtol=2e-7, atol=0)
    ncalls = np.array([int(m) for m in re.findall(r"ncalls= (\d+) at ti=", stdout)])
    if loop == "gsl":
        np.testing.assert_array_equal(ncalls, g["gsl_ncalls"])


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as G
    G.build()


@pytest.mark.gpu
@pytest.mark.parametrize("case", RUN_CASES)
def test_dmdh_run_reproduces_the_reference_run(case, built, tmp_path, capfd):
    from denmat_dynm_development_gb300 import host
    src = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(src, "golden.npz")))
    rundir = str(tmp_path / case)
    os.makedirs(rundir)
    shutil.copy(os.path.join(src, "param.in"), rundir)
    shutil.copytree(os.path.join(src, "ldbd_data"), os.path.join(rundir, "ldbd_data"))
    capfd.readouterr()
    host.run(rundir, "f64")
    check_run_dir(rundir, g, capfd.readouterr().out)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["nb2_eimp_B", "nb2_holes_eq"])
def test_dmdh_run_euler_reproduces_the_reference_run(case, built, tmp_path, capfd):
    """alg_ode_method = euler: DMD's evolve_euler loop (the tau report at its first step comes from
    the same state as evolve_gsl's)"""
    from denmat_dynm_development_gb300 import host
    src = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(src, "golden.npz")))
    rundir = str(tmp_path / case)
    os.makedirs(rundir)
    with open(os.path.join(src, "param.in")) as f:
        text = f.read()
    assert "alg_ode_method = rkf45\n" in text
    with open(os.path.join(rundir, "param.in"), "w") as f:
        f.write(text.replace("alg_ode_method = rkf45\n", "alg_ode_method = euler\n"))
    shutil.copytree(os.path.join(src, "ldbd_data"), os.path.join(rundir, "ldbd_data"))
    capfd.readouterr()
    host.run(rundir, "f64")
    check_run_dir(rundir, g, capfd.readouterr().out, loop="euler")


def check_tau_only_dir(rundir, g):
    """compute_tau_only: the S files hold the t0 line only, the tau files equal the reference's at t0,
    and no step was taken (no restart state)"""
    sz = read_s_file(os.path.join(rundir, "sz_elec_tot.out"))
    assert sz.shape == (1, 3)
    np.testing.assert_allclose(sz[0], g["gsl_sz"][0], rtol=1e-12, atol=0)
    names = sorted(f for f in os.listdir(rundir) if f.startswith("tau_") and f.endswith("_tot.out"))
    assert names == [str(n) for n in g["gsl_tau_names"]]
    for n, text in zip(names, g["gsl_tau_text"]):
        with open(os.path.join(rundir, n)) as f:
            np.testing.assert_allclose(tau_numbers(f.read()), tau_numbers(str(text)), rtol=2e-7, atol=0)
    assert not os.path.exists(os.path.join(rundir, "restart", "denmat_restart.bin"))


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["nb2_holes_eq", "nb4_eimp_B"])
def test_dmdh_run_compute_tau_only(case, built, tmp_path):
    """compute_tau_only = 1: the initial S line and the lifetimes at t0, then no evolution
    (DensityMatrix_Dynamics.h:72-75, main.cpp:79)"""
    from denmat_dynm_development_gb300 import host
    src = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(src, "golden.npz")))
    rundir = str(tmp_path / case)
    os.makedirs(rundir)
    with open(os.path.join(src, "param.in")) as f:
        text = f.read()
    with open(os.path.join(rundir, "param.in"), "w") as f:
        f.write(text + "compute_tau_only = 1\n")
    shutil.copytree(os.path.join(src, "ldbd_data"), os.path.join(rundir, "ldbd_data"))
    host.run(rundir, "f64")
    check_tau_only_dir(rundir, g)


def check_band_columns(rundir, g):
    """print_tot_band = 1: every column of the S_z file (time, total, one per band, amplitude)
    against the reference's run with the same flag"""
    with open(os.path.join(rundir, "sz_elec_tot.out")) as f:
        got = np.array([[float(x) for x in line.split()] for line in f if line.strip() and not line.startswith("#")])
    ref = g["bands_gsl_sz"]
    assert got.shape == ref.shape, (got.shape, ref.shape)
    np.testing.assert_allclose(got[:, 0], ref[:, 0], rtol=1e-13)
    for c in range(1, ref.shape[1]):
        assert np.abs(got[:, c] - ref[:, c]).max() < 1e-10 * np.abs(ref[:, c]).max(), c


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["nb2_eimp_B", "nb4_eimp_B"])
def test_dmdh_run_band_columns(case, built, tmp_path):
    """print_tot_band = 1 (observable.h:376-378): the S files carry each band's share of the total"""
    from denmat_dynm_development_gb300 import host
    src = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(src, "golden.npz")))
    rundir = str(tmp_path / case)
    os.makedirs(rundir)
    with open(os.path.join(src, "param.in")) as f:
        text = f.read()
    with open(os.path.join(rundir, "param.in"), "w") as f:
        f.write(text + "print_tot_band = 1\n")
    shutil.copytree(os.path.join(src, "ldbd_data"), os.path.join(rundir, "ldbd_data"))
    host.run(rundir, "f64")
    check_band_columns(rundir, g)


REF_BIN = os.path.join(os.path.dirname(GOLDEN), os.pardir, "oracle", "_ref", "dmd_ref")


@pytest.mark.skipif(not os.path.exists(REF_BIN), reason="the reference program is built only where its sources are")
def test_checkers_accept_the_reference_runs(tmp_path):
    """The checkers above, applied to the reference program's own run directories for the same
    inputs (evolve_gsl, evolve_euler, compute_tau_only, print_tot_band), accept them: what the GPU
    tests hold dmdh_run to is exactly what the reference writes."""
    import subprocess

    def ref_run(case, mode, edit=lambda t: t):
        d = tmp_path / ("%s_%s_%d" % (case, mode, len(os.listdir(str(tmp_path)))))
        shutil.copytree(os.path.join(GOLDEN, case, "ldbd_data"), str(d / "ldbd_data"))
        with open(os.path.join(GOLDEN, case, "param.in")) as f:
            (d / "param.in").write_text(edit(f.read()))
        args = [REF_BIN, mode] + (["o"] if mode == "dump" else [])
        if mode == "dump":
            os.makedirs(str(d / "o"))
        p = subprocess.run(args, cwd=str(d), capture_output=True, text=True)
        assert p.returncode == 0, p.stderr[-2000:]
        return str(d), p.stdout, dict(np.load(os.path.join(GOLDEN, case, "golden.npz")))

    for case in RUN_CASES:
        d, out, g = ref_run(case, "gsl")
        check_run_dir(d, g, out)
    for case in ["nb2_eimp_B", "nb2_holes_eq"]:
        d, out, g = ref_run(case, "euler", lambda t: t.replace("alg_ode_method = rkf45\n", "alg_ode_method = euler\n"))
        check_run_dir(d, g, out, loop="euler")
    for case in ["nb2_holes_eq", "nb4_eimp_B"]:
        d, out, g = ref_run(case, "dump", lambda t: t + "compute_tau_only = 1\n")
        check_tau_only_dir(d, g)
    for case in ["nb2_eimp_B", "nb4_eimp_B"]:
        d, out, g = ref_run(case, "gsl", lambda t: t + "print_tot_band = 1\n")
        check_band_columns(d, g)
