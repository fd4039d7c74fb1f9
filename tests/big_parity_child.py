"""Child process of test_gpu_big_parity.py: parity at the benchmarked sizes.

Runs in a fresh interpreter so that the oracle's worker processes (forked, DMD's MPI pair split)
start before this process makes any CUDA call. Prints one JSON line with the relative errors:

  * one RHS of the GaAs-like 9.7M-pair workload (nb = 2, nk = 20k, e-ph + e-imp) at t = 3 fs on its
    initial state, GPU (f64 and f64x) against the oracle's RHS split over all host cores;
  * 200 RK4 steps (dt = 1 fs) of the Si-like nk = 500 system (68,971 pairs), GPU f64 and f64x
    against the oracle's RK4 over the same split RHS, state and S_z at the end.

The initial states come from the oracle's restatement of the reference's set-up.
"""
import json
import math
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from denmat_dynm_development_gb300 import ldbd_synth as S  # noqa: E402
from denmat_dynm_development_gb300 import units as U  # noqa: E402
from oracle import oracle as O  # noqa: E402


def workload(name):
    cfg = S.WORKLOADS[name]
    frac = 1e-4 if cfg.eimp_sigma_mev is not None else None
    st, P1, P2, _, _ = S.generate_arrays(cfg, fold_fraction=frac, procs=min(16, os.cpu_count() or 1))
    e = np.ascontiguousarray(st.e)
    f = O.fermi(st.T, (st.mu / U.eV) * U.eV, e)
    dm0 = O.dm_bpert(st.s, e, f, st.T, np.array([0.0, 0.0, 0.1 * U.Tesla2au]), 0.0, 0)
    nk_full = float(st.n) ** 3
    s = O.from_arrays(nk=st.cfg.nk, nb_dm=st.cfg.nb, bstart=0, bend=st.cfg.nb, e_dm=e, f_dm=f, k1st=st.k1,
                      k2nd=st.k2, P1=P1, P2=P2, prefac_eph=2 * math.pi / nk_full, dm0=dm0, smat=st.s,
                      ob_prefac=(1.0 / nk_full) / (st.V * U.bohr2cm ** 3))
    return st, s


def rk4_step(f, t, y, h):
    k1 = f(t, y)
    k2 = f(t + 0.5 * h, y + (0.5 * h) * k1)
    k3 = f(t + 0.5 * h, y + (0.5 * h) * k2)
    k4 = f(t + h, y + h * k3)
    return y + (h / 6.0) * (((k1 + 2.0 * k2) + 2.0 * k3) + k4)


def gpu(st, s, prec):
    from denmat_dynm_development_gb300.dmd import LindbladGPU
    return LindbladGPU(nk=s.nk, nb_dm=s.nb_dm, bstart=0, bend=s.nb_dm, e_dm=s.e_dm, k1st=s.k1st, k2nd=s.k2nd,
                       P1=s.P1, P2=s.P2, prefac_eph=s.prefac_eph, picture=0, expt=1, precision=prec)


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def main():
    O.build()
    O._setup_prototypes()
    ncpu = os.cpu_count() or 1
    out = {}
    # ---- oracle side first (forks), no CUDA yet -------------------------------------------------
    st_big, s_big = workload("gaas_nk20k")
    t = 3.0 * U.fs
    y_big = O.y_of(s_big.dm0)
    par = O.ParallelRHS(s_big, ncpu)
    try:
        ref_big = par(t, y_big)
    finally:
        par.close()
    st_c0, s_c0 = workload("si_nk500")
    y_c0 = O.y_of(s_c0.dm0)
    h, nsteps = 1.0 * U.fs, 200  # (h is also the step of the host-driver check below)
    par = O.ParallelRHS(s_c0, ncpu)
    try:
        yo, tt = y_c0.copy(), 0.0
        for _ in range(nsteps):
            yo = rk4_step(par, tt, yo, h)
            tt += h
    finally:
        par.close()
    sz_o = O.measure(s_c0, yo, tt, 2)
    # ---- GPU ------------------------------------------------------------------------------------
    for prec in ("f64", "f64x"):
        with gpu(st_big, s_big, prec) as g:
            out["rhs_gaas_nk20k_" + prec] = rel(g.func(t, y_big), ref_big)
            if prec == "f64":  # the host RK4 driver over the callback (threaded stage loops at this size)
                from denmat_dynm_development_gb300 import host as HL
                yh = np.ascontiguousarray(y_big, dtype=np.float64).copy()
                HL.rk4_func(g, t, h, 2, yh, np.zeros(5 * yh.size))
                g.set_state(t, y_big)
                g.rk4(h, 2)
                _, yd = g.get_state()
                out["host_rk4_vs_device_gaas_nk20k"] = rel(yh, yd)
        with gpu(st_c0, s_c0, prec) as g:
            g.set_state(0.0, y_c0)
            g.rk4(h, nsteps)
            _, yg = g.get_state()
            out["rk4_si_nk500_200_" + prec] = rel(yg, yo)
            sm = np.ascontiguousarray(st_c0.s[:, 2, :])
            g.set_observable(0, sm, s_c0.f_dm, s_c0.ob_prefac)
            out["sz_si_nk500_200_" + prec] = abs(g.measure(0)[0] - sz_o[0]) / abs(sz_o[0])
    out["npair_gaas_nk20k"] = int(s_big.npair)
    out["npair_si_nk500"] = int(s_c0.npair)
    out["oracle_processes"] = ncpu
    print("RESULT " + json.dumps(out))


if __name__ == "__main__":
    main()
