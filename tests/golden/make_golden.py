"""Generate the golden fixtures under tests/golden/<case>/ from the reference's own code.

Run in a container that has the reference sources (it builds oracle/_ref/dmd_ref with
oracle/Makefile.ref first):

    python tests/golden/make_golden.py [--ref <reference checkout>/src_v4.5.7]

(the default is $DMD_REFERENCE_ROOT/src_v4.5.7, DMD_REFERENCE_ROOT defaulting to /root/reference)

For every case it writes a small synthetic DMD input (param.in + ldbd_data/ from the package's
seeded generator) and runs the shim-built reference program on it:
  * dump  -- setup arrays (initial density matrix, H_BS, occupations);
  * rhs   -- func / evolve_driver / evolve_coh on three states;
  * rk4   -- 40 classic RK4 steps through DMD's func, S_z every 5 steps;
  * gsl   -- DMD's own evolve_gsl (RKF45) for 20 output intervals (S_z file + restart state, and the
             tau files of its report_tau at t0);
  * euler -- DMD's own evolve_euler for 20 steps of tstep (S_z file + restart state);
  * bands (two cases) -- evolve_gsl again with print_tot_band = 1 (S_z file with per-band columns);
  * restart (three cases) -- the set-up dump again with restart = 1 on the state and time that
             evolve_gsl wrote: initial state, t0, chemical potentials and, with alg_ddmdteq, f_eq
             and the equilibrium drift recomputed from the restart state; then compute + report_tau
             there (the tau files at t0 != 0);
  * pee   -- (e-e cases) the operators rebuilt on the three states by reset_scatt: screening density
             from the state, P = P_eph (+ P_eimp) + scale_ee P_ee(rho).
The e-e cases rebuild P_ee on every RHS evaluation (eeMode = Pee_update, freq_update_ee_model < 0),
so their rhs / rk4 / gsl / euler records include the rebuild.
The outputs are stored in golden.npz next to the inputs. Nothing here runs at test time.
"""
from __future__ import annotations

import argparse
import os
import re
import shutil
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from denmat_dynm_development_gb300 import units  # noqa: E402
from denmat_dynm_development_gb300.ldbd_synth import SynthConfig, make_ldbd  # noqa: E402

FS = None

# e-e model keys of param.in (parameters.cpp:192-231): rebuilt from rho on every RHS evaluation
EE_COMMON = {"eeMode": "Pee_update", "scrMode": "medium", "freq_update_ee_model": -1,
             "freq_update_eimp_model": -1, "epsilon_background": 12.9}

CASES = {
    # e-ph only, nb=2, S_z perturbation, interaction picture
    "nb2_eph": dict(cfg=SynthConfig(nk=40, nb=2, seed=11, de_pair_mev=60.0), param=dict(Bpert_T=(0, 0, 0.1))),
    # e-ph + e-imp (D1 files), B field along x -> coherent precession term
    "nb2_eimp_B": dict(cfg=SynthConfig(nk=40, nb=2, seed=12, de_pair_mev=60.0, eimp_sigma_mev=5.0),
                       param=dict(Bpert_T=(0, 0, 0.1), B_T=(2.0, 0, 0), eimp_fraction=0.05)),
    # nb=4 (two spin pairs), e-imp, B field
    "nb4_eimp_B": dict(cfg=SynthConfig(nk=16, nb=4, seed=13, de_pair_mev=60.0, eimp_sigma_mev=5.0),
                       param=dict(Bpert_T=(0.05, 0, 0.1), B_T=(0.5, 0.3, 0), eimp_fraction=0.05)),
    # Schrodinger picture without P(t) phases
    "nb2_schrod": dict(cfg=SynthConfig(nk=30, nb=2, seed=14, de_pair_mev=60.0),
                       param=dict(Bpert_T=(0, 0, 0.1), B_T=(0, 1.0, 0),
                                  extra={"alg_picture": "schrodinger", "alg_expt": 0})),
    # density matrix with 4 bands, e-ph window on the upper 2 (trunc_copy / set_mat path)
    "nb2_window": dict(cfg=SynthConfig(nk=24, nb=2, seed=15, de_pair_mev=60.0, extra_bands=2),
                       param=dict(Bpert_T=(0.1, 0, 0.05), B_T=(0, 0, 1.0))),
    # carrier density given (mu by bisection, electron.h:141-160) and the equilibrium drift
    # subtracted (alg_ddmdteq: set_dm_eq + compute_ddmdt_eq), e-imp, B field
    "nb2_carrier_eq": dict(cfg=SynthConfig(nk=40, nb=2, seed=16, de_pair_mev=60.0, eimp_sigma_mev=5.0),
                           param=dict(Bpert_T=(0, 0, 0.1), B_T=(0.7, 0, 0), eimp_fraction=0.05,
                                      extra={"alg_ddmdteq": 1}),
                           carrier_scale=1.7),
    # linearized master equation (alg_linearize: L_sc operators built from P and f_eq), e-imp, B field
    "nb2_linear": dict(cfg=SynthConfig(nk=40, nb=2, seed=18, de_pair_mev=60.0, eimp_sigma_mev=5.0),
                       param=dict(Bpert_T=(0, 0, 0.1), B_T=(0.5, 0, 0), eimp_fraction=0.05,
                                  extra={"alg_linearize": 1}),
                       carrier_scale=1.3),
    # nb = 4 linearized, Schrodinger picture without phases
    "nb4_linear": dict(cfg=SynthConfig(nk=16, nb=4, seed=19, de_pair_mev=60.0),
                       param=dict(Bpert_T=(0.05, 0, 0.1), B_T=(0, 0.4, 0),
                                  extra={"alg_linearize": 1, "alg_picture": "schrodinger", "alg_expt": 0})),
    # e-e scattering rebuilt from rho on every RHS (Pee_update), Debye screening updated from rho,
    # e-imp folded in, B field; a ball of k-points on the mesh so that k1 + k3 - k2 is mostly present
    "ee_nb2_debye": dict(cfg=SynthConfig(nk=40, nb=2, seed=31, de_pair_mev=60.0, eimp_sigma_mev=5.0, nwannier=4,
                                         kball=True),
                         param=dict(Bpert_T=(0, 0, 0.1), B_T=(0.8, 0, 0), eimp_fraction=0.05,
                                    extra=dict(EE_COMMON, scrFormula="debye", update_screening=1))),
    # exchange term (ee_antisymmetry), Bechstedt screening, Schrodinger picture without phases
    "ee_nb2_bechstedt_anti": dict(cfg=SynthConfig(nk=32, nb=2, seed=32, de_pair_mev=60.0, nwannier=3, kball=True),
                                  param=dict(Bpert_T=(0.05, 0, 0.1), B_T=(0, 0.6, 0),
                                             extra=dict(EE_COMMON, scrFormula="Bechstedt", update_screening=1,
                                                        ee_antisymmetry=1, meff_screening=0.3,
                                                        alg_picture="schrodinger", alg_expt=0))),
    # nb = 4, unscreened Coulomb (Gamma skipped), screening not updated
    "ee_nb4_unscreened": dict(cfg=SynthConfig(nk=16, nb=4, seed=33, de_pair_mev=60.0, nwannier=6, kball=True),
                              param=dict(Bpert_T=(0.05, 0, 0.1), B_T=(0.5, 0.3, 0),
                                         extra=dict(EE_COMMON, scrFormula="unscreened", update_screening=0))),
    # static RPA screening (the reference's default scrFormula) with the screening density updated
    "ee_nb2_rpa": dict(cfg=SynthConfig(nk=36, nb=2, seed=34, de_pair_mev=60.0, nwannier=4, kball=True),
                       param=dict(Bpert_T=(0, 0.05, 0.1), B_T=(0, 0, 0.7),
                                  extra=dict(EE_COMMON, scrFormula="RPA", update_screening=1))),
    # static RPA, nb = 4, exchange term
    "ee_nb4_rpa_anti": dict(cfg=SynthConfig(nk=14, nb=4, seed=35, de_pair_mev=60.0, nwannier=6, kball=True),
                            param=dict(Bpert_T=(0.05, 0, 0.1), B_T=(0.3, 0, 0.2),
                                       extra=dict(EE_COMMON, scrFormula="RPA", update_screening=1,
                                                  ee_antisymmetry=1))),
    # linearized master equation with the e-e source (add_Lsc_contrib("ee"): P_ee at f_eq and the P3-P6
    # terms), Debye screening from f_eq, e-imp, B field
    "ee_nb2_linear": dict(cfg=SynthConfig(nk=40, nb=2, seed=36, de_pair_mev=60.0, eimp_sigma_mev=5.0, nwannier=4,
                                          kball=True),
                          param=dict(Bpert_T=(0, 0, 0.1), B_T=(0.6, 0, 0), eimp_fraction=0.05,
                                     extra=dict(EE_COMMON, scrFormula="debye", update_screening=1, alg_linearize=1)),
                          carrier_scale=1.3),
    # linearized, nb = 4, static RPA, exchange term (P3/P4 skipped, P_ee doubled in Lscij)
    "ee_nb4_linear_rpa_anti": dict(cfg=SynthConfig(nk=14, nb=4, seed=37, de_pair_mev=60.0, nwannier=6, kball=True),
                                   param=dict(Bpert_T=(0.05, 0, 0.1), B_T=(0.3, 0, 0.2),
                                              extra=dict(EE_COMMON, scrFormula="RPA", update_screening=1,
                                                         ee_antisymmetry=1, alg_linearize=1))),
    # linearized, P_ee fixed at equilibrium (no P3-P6), Bechstedt, screening density of the set-up
    "ee_nb2_linear_fixed": dict(cfg=SynthConfig(nk=32, nb=2, seed=38, de_pair_mev=60.0, nwannier=3, kball=True),
                                param=dict(Bpert_T=(0.05, 0, 0.1), B_T=(0, 0.6, 0),
                                           extra=dict(EE_COMMON, eeMode="Pee_fixed_at_eq", scrFormula="Bechstedt",
                                                      update_screening=0, meff_screening=0.3, alg_linearize=1))),
    # dynamic screening in the plasmon-pole approximation (dynamic_screening = ppa, Godby-Needs: the RPA
    # sums at zero and at i * eppa, eppa the plasma frequency of the set-up density), vq(q, w) per
    # matrix element at the mean energy transfer
    "ee_nb2_rpa_ppa": dict(cfg=SynthConfig(nk=36, nb=2, seed=41, de_pair_mev=60.0, nwannier=4, kball=True),
                           param=dict(Bpert_T=(0, 0.05, 0.1), B_T=(0, 0, 0.7),
                                      extra=dict(EE_COMMON, scrFormula="RPA", update_screening=1,
                                                 dynamic_screening="ppa"))),
    # Hybertsen-Louie plasmon pole, nb = 4, exchange term (the exchange factor vq(k1 - k4, w_ex) as
    # the reference applies it), smearing of the real frequency 0.5 T (the default)
    "ee_nb4_rpa_ppa_hl_anti": dict(cfg=SynthConfig(nk=14, nb=4, seed=42, de_pair_mev=60.0, nwannier=6, kball=True),
                                   param=dict(Bpert_T=(0.05, 0, 0.1), B_T=(0.3, 0, 0.2),
                                              extra=dict(EE_COMMON, scrFormula="RPA", update_screening=1,
                                                         dynamic_screening="ppa", ppamodel="hl",
                                                         ee_antisymmetry=1))),
    # Godby-Needs with a given plasmon energy and smearing, the two-frequency interaction
    # (dynamic_screening_ee_two_freqs: |vq| geometric mean, mean phase), exchange term
    "ee_nb2_ppa_twofreq_anti": dict(cfg=SynthConfig(nk=32, nb=2, seed=43, de_pair_mev=60.0, nwannier=3, kball=True),
                                    param=dict(Bpert_T=(0.05, 0, 0.1), B_T=(0, 0.6, 0),
                                               extra=dict(EE_COMMON, scrFormula="RPA", update_screening=0,
                                                          dynamic_screening="ppa", eppa_screening=0.002,
                                                          smearing_screening=0.004,
                                                          dynamic_screening_ee_two_freqs=1,
                                                          ee_antisymmetry=1))),
    # e-e with the equilibrium drift subtracted (alg_ddmdteq): the set-up rebuilds P_ee at rho_eq (its
    # screening density from rho_eq) and the drift is the RHS there; the rebuilds before every RHS then
    # use rho, the drift stays fixed; carrier density given, e-imp folded in
    "ee_nb2_rpa_ddmdteq": dict(cfg=SynthConfig(nk=36, nb=2, seed=45, de_pair_mev=60.0, eimp_sigma_mev=5.0, nwannier=4,
                                               kball=True),
                               param=dict(Bpert_T=(0, 0, 0.1), B_T=(0.5, 0, 0), eimp_fraction=0.05,
                                          extra=dict(EE_COMMON, scrFormula="RPA", update_screening=1,
                                                     alg_ddmdteq=1)),
                               carrier_scale=1.4),
    # sparse operators (alg_sparseP): 70 % of every pair's P1 / P2 elements zeroed, nb = 4, B field;
    # the reference contracts the stored elements with sparse_zgemm (e-ph only: the reference refuses
    # ab-initio e-imp with sparse P)
    "nb4_sparse": dict(cfg=SynthConfig(nk=16, nb=4, seed=41, de_pair_mev=60.0),
                       param=dict(Bpert_T=(0.05, 0, 0.1), B_T=(0.4, 0, 0.3), extra={"alg_sparseP": 1}),
                       zero_fraction=0.7),
    # the same for nb = 2 with half the elements zeroed, Schrodinger picture without phases
    "nb2_sparse": dict(cfg=SynthConfig(nk=40, nb=2, seed=42, de_pair_mev=60.0),
                       param=dict(Bpert_T=(0, 0, 0.1), B_T=(0, 0.8, 0),
                                  extra={"alg_sparseP": 1, "alg_picture": "schrodinger", "alg_expt": 0}),
                       zero_fraction=0.5),
    # two valence bands below the e-ph window (holes: nv_dm = 2), equilibrium drift subtracted
    "nb2_holes_eq": dict(cfg=SynthConfig(nk=24, nb=2, seed=17, de_pair_mev=60.0, extra_bands=2, nv=2),
                         param=dict(Bpert_T=(0.1, 0, 0.05), B_T=(0, 0, 1.0), extra={"alg_ddmdteq": 1})),
}

# cases whose set-up is also recorded in restart mode (restart = 1 on the files evolve_gsl wrote)
RESTART_CASES = ("nb2_eimp_B", "nb2_carrier_eq", "nb2_holes_eq")
# cases run once more with print_tot_band = 1 (per-band columns in the S files); without valence
# bands only: with bStart > 0 the reference scales its band columns at tot_band[i - bStart] for
# i from 0 (observable.h:357-358), outside the array
BAND_CASES = ("nb2_eimp_B", "nb4_eimp_B")


def run(ref_bin, d, *args):
    shutil.rmtree(os.path.join(d, "restart"), ignore_errors=True)
    for f in os.listdir(d):
        if f.endswith(".out") and f != "ref.out":
            os.remove(os.path.join(d, f))
    p = subprocess.run([ref_bin] + list(args), cwd=d, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("reference run failed: %s\n%s" % (args, p.stdout[-3000:] + p.stderr[-3000:]))
    return p.stdout


def read_s_file(path):
    rows = []
    with open(path) as f:
        for line in f:
            if line.startswith("#"):
                continue
            v = line.split()
            if len(v) >= 3:
                rows.append([float(v[0]), float(v[1]), float(v[2])])
    return np.array(rows)


def make_case(name, spec, ref_bin, outroot):
    d = os.path.join(outroot, name)
    shutil.rmtree(d, ignore_errors=True)
    os.makedirs(d)
    cfg = spec["cfg"]
    info = make_ldbd(d, cfg, tstep_fs=1.0, tend_fs=20.0, **spec["param"])
    if spec.get("zero_fraction"):  # structural zeros, the same positions in P1 and P2 of a pair
        rng = np.random.default_rng([cfg.seed, 7])
        nb4 = cfg.nb ** 4
        paths = [os.path.join(d, "ldbd_data", "ldbd_P%d_lindblad.bin" % m) for m in (1, 2)]
        P = [np.fromfile(q, dtype=np.complex128).reshape(-1, nb4) for q in paths]
        mask = rng.random(P[0].shape) < spec["zero_fraction"]
        for q, a in zip(paths, P):
            a[mask] = 0.0
            a.tofile(q)
    if spec.get("carrier_scale"):
        # an electron density carrier_scale times the one at the generator's mu, in cm^-3
        e = np.fromfile(os.path.join(d, "ldbd_data", "ldbd_ek.bin")).reshape(cfg.nk, -1)[:, cfg.nv:]
        n_bvk = float((1.0 / (np.exp((e - info.mu) / info.temperature) + 1.0)).sum()) * spec["carrier_scale"]
        cd = n_bvk / (info.nk_full * info.cell_volume) / units.bohr2cm ** 3
        with open(os.path.join(d, "param.in"), "a") as f:
            f.write("carrier_density = %.17g\n" % cd)
    tmp = os.path.join(d, "_run")
    os.makedirs(tmp)
    shutil.copytree(os.path.join(d, "ldbd_data"), os.path.join(tmp, "ldbd_data"))
    shutil.copy(os.path.join(d, "param.in"), tmp)
    out = {}
    # dump
    os.makedirs(os.path.join(tmp, "o"), exist_ok=True)
    run(ref_bin, tmp, "dump", "o")
    meta = {}
    with open(os.path.join(tmp, "o", "meta.txt")) as f:
        for line in f:
            k, v = line.split()
            meta[k] = float(v)
    nk, nbdm = int(meta["nk"]), int(meta["nb_dm"])
    out["meta_keys"] = np.array(list(meta.keys()))
    out["meta_vals"] = np.array(list(meta.values()))
    out["dm0"] = np.fromfile(os.path.join(tmp, "o", "dm0.bin"), dtype=np.complex128).reshape(nk, nbdm * nbdm)
    out["e_dm"] = np.fromfile(os.path.join(tmp, "o", "e_dm.bin")).reshape(nk, nbdm)
    out["f_dm"] = np.fromfile(os.path.join(tmp, "o", "f_dm.bin")).reshape(nk, nbdm)
    nbw = int(meta["bend"] - meta["bstart"])
    if meta["ddmdteq"] or meta["linearize"]:
        out["f_eq"] = np.fromfile(os.path.join(tmp, "o", "f_eq.bin")).reshape(nk, nbdm)
    if meta["ddmdteq"]:
        out["ddmdt_eq"] = np.fromfile(os.path.join(tmp, "o", "ddmdt_eq.bin"), dtype=np.complex128).reshape(nk, nbw * nbw)
    if meta["linearize"]:
        out["Lscij"] = np.fromfile(os.path.join(tmp, "o", "Lscij.bin"), dtype=np.complex128).reshape(-1, nbw ** 4)
        out["Lscji"] = np.fromfile(os.path.join(tmp, "o", "Lscji.bin"), dtype=np.complex128).reshape(-1, nbw ** 4)
    if meta["has_H"]:
        out["Hcoh"] = np.fromfile(os.path.join(tmp, "o", "Hcoh.bin"), dtype=np.complex128).reshape(nk, nbdm * nbdm)
    ee = bool(meta.get("ee", 0)) and not meta["linearize"]  # (linearized: the e-e term is inside Lscij / Lscji)
    if ee:  # P after set-up: P_eph (+ P_eimp) + scale_ee P_ee at the equilibrium occupations
        out["ee_P1_eq"] = np.fromfile(os.path.join(tmp, "o", "P1.bin"), dtype=np.complex128).reshape(-1, nbw ** 4)
        out["ee_P2_eq"] = np.fromfile(os.path.join(tmp, "o", "P2.bin"), dtype=np.complex128).reshape(-1, nbw ** 4)
    # rhs on three Hermitian states
    rng = np.random.default_rng([cfg.seed, 99])
    fs = 1e-15 * float(np.sqrt((1.0 / 9.10938291e-31) * (1e10 / 0.5291772) ** 2 / (1.0 / 4.35974434e-18)))
    ts = [0.0, 7.3 * fs, 123.4 * fs]
    ys = []
    for t in ts:
        pert = (rng.standard_normal(out["dm0"].shape) + 1j * rng.standard_normal(out["dm0"].shape)) * 1e-3
        dm = (out["dm0"] + pert).reshape(nk, nbdm, nbdm)
        dm = 0.5 * (dm + np.conj(np.swapaxes(dm, 1, 2)))
        ys.append(np.ascontiguousarray(dm.reshape(nk, -1)).view(np.float64).reshape(-1).copy())
    with open(os.path.join(tmp, "rhs_in.bin"), "wb") as f:
        for t, y in zip(ts, ys):
            f.write(np.float64(t).tobytes())
            f.write(y.tobytes())
    if ee:
        run(ref_bin, tmp, "pee", "rhs_in.bin", "o")
        out["pee_P1"] = np.fromfile(os.path.join(tmp, "o", "pee_P1.bin"), dtype=np.complex128).reshape(len(ts), -1, nbw ** 4)
        out["pee_P2"] = np.fromfile(os.path.join(tmp, "o", "pee_P2.bin"), dtype=np.complex128).reshape(len(ts), -1, nbw ** 4)
        out["pee_nfree"] = np.fromfile(os.path.join(tmp, "o", "pee_nfree.bin"))
    run(ref_bin, tmp, "rhs", "rhs_in.bin", "o")
    out["rhs_t"] = np.array(ts)
    out["rhs_y"] = np.stack(ys)
    out["rhs_dydt"] = np.fromfile(os.path.join(tmp, "o", "dydt.bin")).reshape(len(ts), -1)
    out["rhs_eph"] = np.fromfile(os.path.join(tmp, "o", "ddmdt_eph.bin")).reshape(len(ts), -1)
    out["rhs_coh"] = np.fromfile(os.path.join(tmp, "o", "ddmdt_coh.bin")).reshape(len(ts), -1)
    # rk4: 40 steps of 1 fs, S_z every 5 steps
    run(ref_bin, tmp, "rk4", "1.0", "40", "5", "o")
    out["rk4_y"] = np.fromfile(os.path.join(tmp, "o", "y_final.bin"))
    out["rk4_sz"] = read_s_file(os.path.join(tmp, "sz_elec_tot.out"))
    # gsl: DMD's evolve_gsl to tend = 20 fs, output every tstep = 1 fs
    log = run(ref_bin, tmp, "gsl")
    out["gsl_sz"] = read_s_file(os.path.join(tmp, "sz_elec_tot.out"))
    out["gsl_ncalls"] = np.array([int(m) for m in re.findall(r"ncalls= (\d+) at ti=", log)])
    out["gsl_y"] = np.fromfile(os.path.join(tmp, "restart", "denmat_restart.bin"))
    # the tau files evolve_gsl wrote at its first step (compute + report_tau at t0), as text
    tau_files = sorted(f for f in os.listdir(tmp) if f.startswith("tau_") and f.endswith("_tot.out"))
    out["gsl_tau_names"] = np.array(tau_files)
    out["gsl_tau_text"] = np.array([open(os.path.join(tmp, f)).read() for f in tau_files])
    if name in BAND_CASES:
        bdir = os.path.join(d, "_bands")
        os.makedirs(bdir)
        shutil.copytree(os.path.join(d, "ldbd_data"), os.path.join(bdir, "ldbd_data"))
        with open(os.path.join(d, "param.in")) as f:
            text = f.read()
        with open(os.path.join(bdir, "param.in"), "w") as f:
            f.write(text + "print_tot_band = 1\n")
        run(ref_bin, bdir, "gsl")
        with open(os.path.join(bdir, "sz_elec_tot.out")) as f:  # every column: t, total, bands, amplitude
            out["bands_gsl_sz"] = np.array([[float(x) for x in line.split()] for line in f
                                            if line.strip() and not line.startswith("#")])
        shutil.rmtree(bdir)
    if name in RESTART_CASES:
        # the reference's set-up with restart = 1 (parameters.cpp:298-309, read_dm_restart
        # DenMat.cpp:301-316) from the state and time its evolve_gsl wrote (write_dm_tofile)
        rdir = os.path.join(d, "_restart")
        os.makedirs(rdir)
        shutil.copytree(os.path.join(d, "ldbd_data"), os.path.join(rdir, "ldbd_data"))
        shutil.copytree(os.path.join(tmp, "restart"), os.path.join(rdir, "restart"))
        with open(os.path.join(d, "param.in")) as f:
            text = f.read()
        assert "restart = 0\n" in text
        with open(os.path.join(rdir, "param.in"), "w") as f:
            f.write(text.replace("restart = 0\n", "restart = 1\n"))
        os.makedirs(os.path.join(rdir, "o"))
        p = subprocess.run([ref_bin, "dump", "o"], cwd=rdir, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("reference restart dump failed:\n" + p.stdout[-3000:] + p.stderr[-3000:])
        rmeta = {}
        with open(os.path.join(rdir, "o", "meta.txt")) as f:
            for line in f:
                k, v = line.split()
                rmeta[k] = float(v)
        out["restart_in_y"] = np.fromfile(os.path.join(rdir, "restart", "denmat_restart.bin"))
        with open(os.path.join(rdir, "restart", "time_restart.dat")) as f:
            out["restart_in_time"] = np.array(f.read())
        out["restart_t0"] = np.float64(rmeta["t0"])
        out["restart_mu"] = np.array([rmeta["mue"], rmeta["muh"]])
        out["restart_dm0"] = np.fromfile(os.path.join(rdir, "o", "dm0.bin"), dtype=np.complex128).reshape(nk, nbdm * nbdm)
        if rmeta["ddmdteq"]:
            out["restart_f_eq"] = np.fromfile(os.path.join(rdir, "o", "f_eq.bin")).reshape(nk, nbdm)
            out["restart_ddmdt_eq"] = np.fromfile(os.path.join(rdir, "o", "ddmdt_eq.bin"),
                                                  dtype=np.complex128).reshape(nk, nbw * nbw)
        # compute + report_tau at the restart time (t0 != 0: the phases and the other line format)
        p = subprocess.run([ref_bin, "tau"], cwd=rdir, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("reference restart tau failed:\n" + p.stdout[-3000:] + p.stderr[-3000:])
        tau_files = sorted(f for f in os.listdir(rdir) if f.startswith("tau_") and f.endswith("_tot.out"))
        out["restart_tau_names"] = np.array(tau_files)
        out["restart_tau_text"] = np.array([open(os.path.join(rdir, f)).read() for f in tau_files])
        shutil.rmtree(rdir)
    # euler: DMD's evolve_euler to tend = 20 fs in steps of tstep = 1 fs
    run(ref_bin, tmp, "euler")
    out["euler_sz"] = read_s_file(os.path.join(tmp, "sz_elec_tot.out"))
    out["euler_y"] = np.fromfile(os.path.join(tmp, "restart", "denmat_restart.bin"))
    np.savez_compressed(os.path.join(d, "golden.npz"), **out)
    shutil.rmtree(tmp)
    return info


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.path.join(os.environ.get("DMD_REFERENCE_ROOT", "/root/reference"),
                                                  "src_v4.5.7"))
    ap.add_argument("--cases", nargs="*", default=list(CASES))
    a = ap.parse_args()
    subprocess.run(["make", "-f", os.path.join(ROOT, "oracle", "Makefile.ref"), "-j8", "REF=" + a.ref], check=True,
                   cwd=ROOT, stdout=subprocess.DEVNULL)
    ref_bin = os.path.join(ROOT, "oracle", "_ref", "dmd_ref")
    outroot = os.path.dirname(os.path.abspath(__file__))
    for name in a.cases:
        info = make_case(name, CASES[name], ref_bin, outroot)
        print(name, "nk=%d nb=%d npair=%d" % (info.nk, info.nb, info.npair))


if __name__ == "__main__":
    main()
