#!/usr/bin/env python
"""Benchmark: RK4 steps/s of DMD's Lindblad density-matrix dynamics on the GaAs-like workload.

Workload (gaas_nk20k): nb = 2 spin-split conduction bands, nk = 20000 k-points, ~9.7M k-pairs
(P1 + P2 = 5.0 GB complex128), e-ph plus an ab-initio-style e-imp term folded into P
(|n_i V_cell| = 1e-4), spin perturbation Bz = 0.1 T, RK4 with dt = 1 fs. Seeded synthetic data
from the package generator (the reference publishes no dataset for this path).

One step = one RK4 step = four RHS evaluations, each streaming all of P once (inputs are larger
than the 129 MB L2, so no flush is needed between steps).

The headline arithmetic is the reference's: plain FP64 (P complex128, FP64 multiply-adds).

  value       RK4 steps/s with the density matrix resident on the GPU (dmd_rk4, CUDA graph); the
              K-step window is timed `--windows` times (CUDA events) and the median is reported,
              with the spread
  e2e         the same metric through the reference-facing GSL callback dmd_func: the host runs
              the RK4 combination in C loops (dmdh_rk4_func) and every RHS call copies y in and
              dydt out (page-locked buffers)
  roofline    k-pair contraction kernel: algorithmic work per launch / its mean event-timed
              duration, against the ceiling that binds it -- the FP64 multiply-add rate measured in
              this process for the FP64 form (its work is FP64 multiply-adds; the HBM fraction is
              reported beside it), the measured HBM copy bandwidth for the other forms
  forms       the other arithmetics of the same contraction on the same workload (f64x: FP32
              pairs; f32 and bf16x2: reduced-precision storage with rho as a deviation from f),
              each with its steps/s, roofline and RHS error against the oracle's FP64 RHS
  cpu_baseline the oracle port of the reference's RHS on this host (test infrastructure): one RK4
              step of the full workload on one core; its first RHS is also the reference the
              forms' errors are measured against

--impl reference runs the CPU restatement of the reference's code path (DMD's MPI pair
decomposition as forked processes over all host cores) on the same workload, config and metric;
its set-up (occupations, initial state) is the oracle's own, so no product library is loaded.
N > 1 GPUs run independent replicas (the path's only exchange is a per-RHS allreduce that this
build does not distribute); value is the sum over ranks of steps/s.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from denmat_dynm_development_gb300 import ldbd_synth as S  # noqa: E402
from denmat_dynm_development_gb300 import units as U  # noqa: E402

METRIC = "RK4 steps/s (plain FP64 Lindblad RHS, k-pair P streamed from HBM)"
UNIT = "RK4 steps/s"


def env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


# ------------------------------------------------------------------------------------------------
# workload
# ------------------------------------------------------------------------------------------------
def build_workload(name, procs, cfg=None, setup="host"):
    """Seeded synthetic workload. setup = "host": occupations and initial state from the product's
    host library; "oracle": from the oracle's restatement of the same set-up (bit-identical, tests),
    for the reference arm, which must not load the product libraries."""
    cfg = S.WORKLOADS[name] if cfg is None else cfg
    frac = 1e-4 if cfg.eimp_sigma_mev is not None else None
    t0 = time.time()
    st, P1, P2, _, _ = S.generate_arrays(cfg, fold_fraction=frac, procs=procs)
    gen_s = time.time() - t0
    if setup == "oracle":
        from oracle import oracle as H
    else:
        from denmat_dynm_development_gb300 import host as H
    T = st.T
    mu = (st.mu / U.eV) * U.eV          # parameters::get round trip
    e = np.ascontiguousarray(st.e)
    f = H.fermi(T, mu, e)
    Bpert = np.array([0.0, 0.0, 0.1 * U.Tesla2au])
    dm0 = H.dm_bpert(st.s, e, f, T, Bpert, 0.0, 0)
    nk_full = float(st.n) ** 3
    V = st.V
    ob_prefac = (1.0 / nk_full) / (V * U.bohr2cm ** 3)
    w = dict(name=name, cfg=cfg, st=st, P1=P1, P2=P2, e=e, f=f, dm0=dm0, T=T, mu=mu, nk_full=nk_full,
             prefac=2 * math.pi / nk_full, ob_prefac=ob_prefac, gen_s=gen_s, frac=frac)
    return w


def algorithmic_bytes(nb, npair, nk, prec_bytes=16):
    """Per RHS evaluation of the pair contraction: P1+P2 once, two int32 indices per pair, the
    per-k vectors read and the per-k sums written."""
    return npair * (2 * nb ** 4 * prec_bytes + 8) + nk * nb * nb * 16 * 2 + nk * nb * 8


def algorithmic_flops(nb, npair):
    """Per RHS evaluation of the pair contraction in Hermitian coordinates: every element of P1 and
    P2 (2 nb^4 complex per pair) enters the forward and the reverse sum once each as a complex x real
    product (2 multiply-adds = 4 flops). (The reference's complex-form GEMVs take twice that.)"""
    return npair * 2 * nb ** 4 * 2 * 4


L2_BYTES = 129e6


def config_of(w):
    """The workload; identical in both arms (the arm's own settings go under "arm")."""
    st = w["st"]
    nb = st.cfg.nb
    pbytes = 2 * st.npair * nb ** 4 * 16
    if pbytes > L2_BYTES:
        l2 = "inputs larger than L2 (P streamed once per RHS: %.2f GB > 129 MB); no flush" % (pbytes / 1e9)
    else:
        l2 = "P (%.1f MB) fits in the 129 MB L2: L2-resident timing, no flush" % (pbytes / 1e6)
    return {"workload": "%s: nb=%d, nk=%d, %d k-pairs (P1+P2 %.2f GB complex128), e-ph%s, Bz_pert 0.1 T, RK4 dt=1 fs"
                        % (w["name"], nb, st.cfg.nk, st.npair, pbytes / 1e9,
                           " + e-imp (|n_i V|=1e-4)" if w["frac"] else ""),
            "nk": st.cfg.nk, "nb": nb, "npair": st.npair, "dt_fs": 1.0, "l2": l2, "parallelism": "replicas"}


# ------------------------------------------------------------------------------------------------
# clocks sampled during the timed region
# ------------------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the sampler is running once its first line arrives; what came before the timed region
            # (idle clocks) is dropped
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.lines = []
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            v = [x.strip() for x in ln.split(",")]
            if len(v) < 9:
                continue
            try:
                sm.append(float(v[1]))
                smax.append(float(v[2]))
            except ValueError:
                continue
            for n, x in zip(names, v[5:9]):
                if x.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(precision):
    """DRAM bytes per pair-kernel launch from the committed ncu summary of this arithmetic, as
    (bytes, npair of the captured workload); scaled by the caller to the benchmarked workload."""
    p = os.path.join(ROOT, "profiles", "pairs_herm_%s_gaas_nk16k.md" % precision)
    try:
        vals = {}
        with open(p) as f:
            for line in f:
                if ":" in line and line.split(":")[0].strip() in ("traffic_bytes_per_launch", "traffic_npair"):
                    vals[line.split(":")[0].strip()] = float(line.split(":")[1])
        return vals["traffic_bytes_per_launch"], vals["traffic_npair"]
    except Exception:
        return None


# ------------------------------------------------------------------------------------------------
# CPU baseline (oracle port) and reference arm
# ------------------------------------------------------------------------------------------------
def oracle_system(w):
    from oracle import oracle as O
    O.build()
    O._setup_prototypes()
    st = w["st"]
    return O, O.from_arrays(nk=st.cfg.nk, nb_dm=st.cfg.nb, bstart=0, bend=st.cfg.nb, e_dm=w["e"], f_dm=w["f"],
                            k1st=st.k1, k2nd=st.k2, P1=w["P1"], P2=w["P2"], prefac_eph=w["prefac"], dm0=w["dm0"],
                            temperature=w["T"], mu=w["mu"], nk_full=w["nk_full"], ob_prefac=w["ob_prefac"])


def rk4_host_step(f, t, y, h):
    """y_{n+1} = y + h/6 (k1 + 2 k2 + 2 k3 + k4) with f(t, y) a host-buffer RHS."""
    k1 = f(t, y)
    k2 = f(t + 0.5 * h, y + (0.5 * h) * k1)
    k3 = f(t + 0.5 * h, y + (0.5 * h) * k2)
    k4 = f(t + h, y + h * k3)
    return y + (h / 6.0) * (((k1 + 2.0 * k2) + 2.0 * k3) + k4)


def cpu_baseline_leg(w, t0=3.0 * U.fs):
    """One RK4 step of the full workload through the oracle's func() on one core (the reference is
    serial per MPI rank): steps/s = 1 / (time of the step). Also returns its first stage,
    f(t0, y0), the FP64 reference the GPU forms' errors are measured against."""
    O, s = oracle_system(w)
    y = O.y_of(w["dm0"])
    h = 1.0 * U.fs
    out = {}

    def f(t, yy):
        r = O.rhs(s, t, yy)
        if "k1" not in out:
            out["k1"] = r
        return r
    t_start = time.perf_counter()
    rk4_host_step(f, t0, y, h)
    dt = time.perf_counter() - t_start
    line = {"value": 1.0 / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "one RK4 step (4 func() evaluations) of the full workload (%d pairs) in %.1f s on one core"
                      % (s.npair, dt)}
    return line, out["k1"], t0, y


def run_reference(args, w):
    O, s = oracle_system(w)
    cores = os.cpu_count() or 1
    par = O.ParallelRHS(s, cores)
    try:
        h = 1.0 * U.fs
        y = O.y_of(w["dm0"])
        t = 0.0
        for _ in range(args.warmup):
            y = rk4_host_step(par, t, y, h)
            t += h
        t0 = time.perf_counter()
        for _ in range(args.steps):
            y = rk4_host_step(par, t, y, h)
            t += h
        el = time.perf_counter() - t0
    finally:
        par.close()
    v = args.steps / el
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_of(w),
            "arm": {"parallelism": "%d forked CPU processes (DMD's MPI pair split, allreduce by summation)" % cores,
                    "setup": "oracle restatement of the reference's set-up (fermi, compute_dm_Bpert_1st, init_dm)"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "%d RK4 steps of the full workload, pairs split over %d processes as DMD's "
                                       "MPI ranks split them, allreduce by summation" % (args.steps, cores)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ------------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------------
def batch_states(w, nrhs, seed=7):
    """nrhs initial states sharing the workload's P: first-order spin polarisations along x, y, z
    (0.1 T, electron.cpp:62-98) in turn, each with its own random Hermitian 1e-4 deviation standing
    in for a pump with a random Jones vector."""
    from denmat_dynm_development_gb300 import host as H
    st = w["st"]
    rng = np.random.default_rng(seed)
    out = []
    for q in range(nrhs):
        B = np.zeros(3)
        B[q % 3] = 0.1 * U.Tesla2au
        d = H.dm_bpert(st.s, w["e"], w["f"], w["T"], B, 0.0, 0).reshape(st.cfg.nk, st.cfg.nb, st.cfg.nb)
        x = 1e-4 * (rng.standard_normal(d.shape) + 1j * rng.standard_normal(d.shape)) * w["f"][:, :, None]
        d = d + 0.5 * (x + np.conj(np.swapaxes(x, 1, 2)))
        out.append(np.ascontiguousarray(d.reshape(st.cfg.nk, -1)).view(np.float64).reshape(-1))
    return np.concatenate(out)


def run_gpu_batched(args, w):
    """Batched form: args.nrhs states share P; value = states x RK4 steps per second."""
    from denmat_dynm_development_gb300.dmd import LindbladGPU
    st = w["st"]
    nb = st.cfg.nb
    R = args.nrhs
    prec = args.precision if args.precision in ("f32", "bf16x2") else "bf16x2"
    tc = prec == "bf16x2" and nb in (2, 4) and os.environ.get("DMD_BATCH_TC", "1") != "0"
    g = LindbladGPU(nk=st.cfg.nk, nb_dm=nb, bstart=0, bend=nb, e_dm=w["e"], k1st=st.k1, k2nd=st.k2, P1=w["P1"],
                    P2=w["P2"], prefac_eph=w["prefac"], picture=0, expt=1, precision=prec, f_ref=w["f"], nrhs=R)
    h = 1.0 * U.fs
    g.set_state(0.0, batch_states(w, R))
    shape = g.autotune(3)
    g.rk4(h, args.warmup)
    clk = ClockSampler(0)
    clk.start()
    g.sync()
    l0 = g.launches
    g.timer_start()
    g.rk4(h, args.steps)
    ms = g.timer_stop()
    g.sync()
    clocks = clk.stop()
    launches = g.launches - l0
    g.set_profiling(True)
    g.rk4(h, 2)
    pair_ms, pair_n = g.profile(1)
    prep_ms, prep_n = g.profile(0)
    fin_ms, fin_n = g.profile(2)
    g.set_profiling(False)
    pbytes = g.pair_bytes
    g.close()
    ms_per_step = ms / args.steps
    peak, peak_kind = measured_peak()
    pair_avg = pair_ms / max(pair_n, 1)
    nk = st.cfg.nk
    if tc:
        # per contraction (packing + Hermitian pass): operator blocks once from HBM, the r coordinates
        # in (FP32) and as bf16 hi + lo blocks out and back in, the sums out
        nb2 = nb * nb
        nmb = (R + 127) // 128
        ngroups = (nk + 32 // nb2 - 1) // (32 // nb2)  # column groups of 32 / nb^2 k-points
        bpl = pbytes + R * nk * nb2 * 4 + 2 * ngroups * nmb * 16384 + R * nk * 2 * nb2 * 16
        flops = (pbytes / 32768) * nmb * 6 * 2.0 * 128 * 256 * 16  # issued MMA flops (padding included)
        kernel, bound = "tensor-core batched k-pair contraction (tcgen05, bf16 hi+lo)", "hbm"
    else:
        bpl = algorithmic_bytes(nb, st.npair, nk, ELEM_BYTES[prec]) + (R - 1) * nk * nb * nb * 16 * 2
        flops = 2.0 * 4 * nb ** 4 * 2 * st.npair * R  # complex x real products of the four sums, per RHS evaluation
        kernel, bound = "batched k-pair contraction (CUDA cores)", "fp32-issue"
    line = {"metric": "ensemble RK4 steps/s (%d states sharing P, batched form)" % R, "value": R * 1e3 / ms_per_step,
            "unit": "state-steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": prec + " (rho as deviation from f)", "data": "synthetic",
            "config": dict(config_of(w), nrhs=R,
                           states="spin polarisation along x/y/z in turn + random 1e-4 deviation"),
            "arm": {"precision": prec, "tensor_cores": tc, "autotuned_shape": shape},
            "roofline": {"bound": bound, "achieved": bpl / (pair_avg * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": bpl / (pair_avg * 1e-3) / 1e9 / peak, "traffic": None, "peak_kind": peak_kind,
                         "kernel": kernel, "avg_launch_ms": pair_avg, "pair_bytes": pbytes,
                         "tflops": flops / (pair_avg * 1e-3) / 1e12,
                         "per_rhs_ms": {"prep": prep_ms / max(prep_n, 1), "contraction": pair_avg,
                                        "finish": fin_ms / max(fin_n, 1)}},
            "clocks": clocks, "gpu_launches": launches}
    print(json.dumps(line))


class Timed:
    """A handle's K-step RK4 window timed with CUDA events on its stream, `windows` times."""

    def __init__(self, g, h, steps, windows, barrier=None):
        self.ms = []
        self.launches = 0
        for i in range(windows):
            if barrier:
                barrier()
            g.sync()
            l0 = g.launches
            g.timer_start()
            g.rk4(h, steps)
            self.ms.append(g.timer_stop())
            g.sync()
            if barrier:
                barrier()
            if i == 0:
                self.launches = g.launches - l0
        self.median = statistics.median(self.ms)

    def spread(self, steps):
        return {"windows": len(self.ms), "ms_per_step_median": self.median / steps,
                "ms_per_step_min": min(self.ms) / steps, "ms_per_step_max": max(self.ms) / steps}


def kernel_profile(g, h, steps):
    """per-kernel event timing of a profiled pass (kernels launched one by one, no graph)"""
    g.set_profiling(True)
    g.rk4(h, steps)
    out = {c: g.profile(i) for i, c in enumerate(("prep", "pairs", "finish"))}
    g.set_profiling(False)
    return {k: v[0] / max(v[1], 1) for k, v in out.items()}, out["pairs"][1]


def roofline_of(prec, nb, npair, nk, pair_ms, peaks, traffic):
    """Roofline of the contraction kernel. FP64: bound by the FP64 multiply-add rate measured in
    this process (its algorithmic flops per launch / the event-timed launch); the HBM fraction of its
    algorithmic bytes is reported beside it. Other forms: HBM."""
    hbm, hbm_kind = peaks["hbm"]
    bpl = algorithmic_bytes(nb, npair, nk, ELEM_BYTES[prec])
    gbs = bpl / (pair_ms * 1e-3) / 1e9
    r = {"kernel": "k-pair contraction (k_pairs_herm, %s)" % prec, "avg_launch_ms": pair_ms, "bytes_per_launch": bpl,
         "traffic": traffic}
    if prec == "f64":
        fl = algorithmic_flops(nb, npair)
        tf = fl / (pair_ms * 1e-3) / 1e12
        r.update({"bound": "fp64", "achieved": tf, "peak": peaks["fp64"], "unit": "TFLOP/s",
                  "frac": tf / peaks["fp64"], "peak_kind": "measured in-process (dmd_peak_fma, FP64 FMA)",
                  "flops_per_launch": fl, "hbm_achieved_gbs": gbs, "hbm_peak_gbs": hbm, "hbm_frac": gbs / hbm,
                  "hbm_peak_kind": hbm_kind,
                  "binding": "FP64 pipe: HBM alone would allow %.3f ms per launch, the measured FP64 rate %.3f ms"
                             % (bpl / (hbm * 1e9) * 1e3, fl / (peaks["fp64"] * 1e12) * 1e3)})
    else:
        r.update({"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                  "peak_kind": hbm_kind})
    return r


def make_handle(w, prec, dev):
    from denmat_dynm_development_gb300.dmd import LindbladGPU
    st = w["st"]
    nb = st.cfg.nb
    return LindbladGPU(nk=st.cfg.nk, nb_dm=nb, bstart=0, bend=nb, e_dm=w["e"], k1st=st.k1, k2nd=st.k2, P1=w["P1"],
                       P2=w["P2"], prefac_eph=w["prefac"], picture=0, expt=1, precision=prec, device=dev,
                       f_ref=w["f"])


def rel_err(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def run_gpu(args, w, rank, world, dist):
    from denmat_dynm_development_gb300.dmd import PinnedArray, peak_fma
    st = w["st"]
    nb = st.cfg.nb
    dev = env_int("LOCAL_RANK", 0)
    h = 1.0 * U.fs
    lead = rank == 0 and world == 1
    # the oracle's CPU leg first (one core, no GPU involved): the CPU baseline and the FP64 reference RHS
    cpu = ref_rhs = None
    if args.cpu_baseline and lead:
        cpu, ref_rhs, t_ref, y_ref = cpu_baseline_leg(w)
    peaks = {"hbm": measured_peak(), "fp64": peak_fma(dev, True), "fp32": peak_fma(dev, False)}
    t_create = time.perf_counter()
    g = make_handle(w, args.precision, dev)
    t_create = time.perf_counter() - t_create  # layout, device conversion and upload of P
    y0 = np.ascontiguousarray(w["dm0"]).view(np.float64).reshape(-1).copy()
    g.set_state(0.0, y0)
    shape = g.autotune(3) if args.autotune else None  # compiled contraction shapes timed, fastest kept
    g.rk4(h, args.warmup)                      # warm-up (also captures the step graph)

    def barrier():
        if dist is not None:
            dist.barrier()
    # ---- timed region: device-resident RK4, the K-step window `windows` times ------------------
    clk = ClockSampler(dev)
    clk.start()
    tm = Timed(g, h, args.steps, args.windows, barrier)
    clocks = clk.stop()
    ms = tm.median
    if dist is not None:
        import torch
        tt = torch.tensor([ms], dtype=torch.float64, device="cuda:%d" % dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    ms_per_step = ms / args.steps
    value = world * 1e3 / ms_per_step
    kms, pair_n = kernel_profile(g, h, max(2, min(args.steps, 10)))
    # ---- end to end through the GSL-callback ABI with host buffers ---------------------------
    e2e = None
    if not args.no_e2e:
        n = y0.size
        from denmat_dynm_development_gb300 import host as HL
        bufs = [PinnedArray(n), PinnedArray(5 * n)]  # y; stage input and k1..k4
        try:
            yv, work = bufs[0].array, bufs[1].array
            _, ycur = g.get_state()
            yv[:] = ycur
            t = 0.0
            HL.rk4_func(g, t, h, 1, yv, work)  # warm-up
            barrier()
            t0 = time.perf_counter()
            HL.rk4_func(g, t, h, args.steps, yv, work)
            el = time.perf_counter() - t0
            t += args.steps * h
            e2e = {"value": world * args.steps / el, "unit": UNIT, "h2d_bytes_per_step": 4 * n * 8,
                   "d2h_bytes_per_step": 4 * n * 8,
                   "path": "host RK4 loop (dmdh_rk4_func) calling the GSL-callback entry dmd_func 4x per step "
                           "from page-locked buffers, stage combinations in host loops; %d steps" % args.steps}
        finally:
            for b in bufs:
                b.free()
    err = rel_err(g.func(t_ref, y_ref), ref_rhs) if ref_rhs is not None else None
    g.close()
    if rank != 0:
        return
    tr = profile_traffic(args.precision)
    traffic = tr[0] * st.npair / tr[1] if tr else None  # the capture's bytes per pair times this workload's
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": DTYPE[args.precision], "data": "synthetic", "config": config_of(w),
            "arm": {"precision": args.precision, "autotuned_shape": shape, "create_s": t_create,
                    "gen_seconds": w["gen_s"]},
            "timing": dict(tm.spread(args.steps), how="CUDA events on the handle's stream around each K-step "
                                                       "window; value from the median window"),
            "roofline": roofline_of(args.precision, nb, st.npair, st.cfg.nk, kms["pairs"], peaks, traffic),
            "kernel_ms_per_step": {k: 4 * v for k, v in kms.items()},
            "peaks": {"hbm_gbs": peaks["hbm"][0], "hbm_kind": peaks["hbm"][1], "fp64_fma_tflops": peaks["fp64"],
                      "fp32_fma_tflops": peaks["fp32"]},
            "e2e": e2e, "clocks": clocks, "gpu_launches": tm.launches}
    if err is not None:
        line["rhs_rel_err_vs_oracle"] = err
    if lead and args.forms:
        line["forms"] = run_forms(args, w, dev, peaks, (t_ref, y_ref, ref_rhs) if ref_rhs is not None else None)
    if lead and args.t1:
        line["t1"] = t1_compare([p for p in ("f64x", "f32", "bf16x2") if p != args.precision] if args.forms
                                else ([args.precision] if args.precision != "f64" else []),
                                args.t1_steps, dev, "si_nk500" if nb == 2 else "mos2_nk2k")
    if cpu is not None:
        line["cpu_baseline"] = cpu
    print(json.dumps(line))


ELEM_BYTES = {"f64": 16, "f64x": 16, "f32": 8, "bf16x2": 8}
DTYPE = {"f64": "f64", "f64x": "f64 (fp32-pair emulated)", "f32": "f32 (P complex64, rho as deviation from f)",
         "bf16x2": "bf16 hi+lo (P 8 B/complex, rho as deviation from f)"}


def run_forms(args, w, dev, peaks, ref):
    """The other arithmetics of the contraction on the same workload: RK4 steps/s (median of 3
    K-step windows), the contraction's roofline, and the RHS error against the oracle's FP64 RHS."""
    st = w["st"]
    nb = st.cfg.nb
    h = 1.0 * U.fs
    y0 = np.ascontiguousarray(w["dm0"]).view(np.float64).reshape(-1).copy()
    out = {}
    for prec in ("f64", "f64x", "f32", "bf16x2"):
        if prec == args.precision:
            continue
        g = make_handle(w, prec, dev)
        try:
            g.set_state(0.0, y0)
            shape = g.autotune(3)
            g.rk4(h, args.warmup)
            tm = Timed(g, h, args.steps, 3)
            kms, _ = kernel_profile(g, h, max(2, min(args.steps, 10)))
            tr = profile_traffic(prec)
            r = {"dtype": DTYPE[prec], "value": 1e3 * args.steps / tm.median, "unit": UNIT,
                 "timing": tm.spread(args.steps), "autotuned_shape": shape,
                 "roofline": roofline_of(prec, nb, st.npair, st.cfg.nk, kms["pairs"], peaks,
                                         tr[0] * st.npair / tr[1] if tr else None),
                 "kernel_ms_per_step": {k: 4 * v for k, v in kms.items()}}
            if ref is not None:
                r["rhs_rel_err_vs_oracle"] = rel_err(g.func(ref[0], ref[1]), ref[2])
            out[prec] = r
        finally:
            g.close()
    return out


def t1_compare(precisions, nsteps, dev, workload):
    """T1 of a small case of the same band count (Si-like nk=500 for nb=2, MoS2-like nk=2000 for
    nb=4; RK4 dt = 1 fs, S_z every 100 steps, exponential fit) from each precision and from the plain
    FP64 GPU path on the same input (the FP64 path itself matches the FP64 oracle's T1 to 1e-10 in the
    GPU tests). The lifetimes compared are the least-squares optimum converged to machine precision
    (tau_conv). The equilibrium drift of f is subtracted (alg_ddmdteq with f_eq = f) so that f is
    stationary."""
    from denmat_dynm_development_gb300.dmd import LindbladGPU
    from denmat_dynm_development_gb300.t1fit import fit_t1
    w = build_workload(workload, 4)
    st = w["st"]
    nb = st.cfg.nb
    y0 = np.ascontiguousarray(w["dm0"]).view(np.float64).reshape(-1).copy()
    idx = np.arange(nb)
    feq = np.zeros((st.cfg.nk, nb, nb), np.complex128)
    feq[:, idx, idx] = w["f"]
    yf = np.ascontiguousarray(feq.reshape(st.cfg.nk, -1)).view(np.float64).reshape(-1).copy()
    out = {}
    eq = None
    t0 = time.perf_counter()
    for prec in ["f64"] + list(precisions):
        g = LindbladGPU(nk=st.cfg.nk, nb_dm=nb, bstart=0, bend=nb, e_dm=w["e"], k1st=st.k1, k2nd=st.k2,
                        P1=w["P1"], P2=w["P2"], prefac_eph=w["prefac"], picture=0, expt=1, precision=prec, device=dev,
                        f_ref=w["f"])
        try:
            if eq is None:
                eq = g.evolve_driver(0.0, yf).view(np.complex128).reshape(st.cfg.nk, nb * nb).copy()
            g.set_ddmdt_eq(eq)
            g.set_state(0.0, y0)
            sz = np.ascontiguousarray(st.s[:, 2, :])
            g.set_observable(0, sz, w["f"], w["ob_prefac"])
            rec = []
            for _ in range(nsteps // 100):
                g.rk4(1.0 * U.fs, 100)
                t, _ = g.get_state()
                rec.append((t,) + g.measure(0))
            out[prec] = np.array(rec)
        finally:
            g.close()
    a = out["f64"]
    fa = fit_t1(a[:, 0], a[:, 1])
    res = {"workload": "%s: nb=%d, nk=%d, %d k-pairs, RK4 dt=1 fs, %d steps, S_z every 100 steps, "
                       "drift of f subtracted" % (workload, nb, st.cfg.nk, st.npair, nsteps),
           "tau_ps_f64": fa.tau_conv, "s_ratio_end": float(a[-1, 1] / a[0, 1]), "fit": "converged least squares"}
    for prec in precisions:
        b = out[prec]
        fb = fit_t1(b[:, 0], b[:, 1])
        res[prec] = {"tau_ps": fb.tau_conv, "rel_err": abs(fb.tau_conv - fa.tau_conv) / abs(fa.tau_conv),
                     "s_rel_err": float(np.abs(b[:, 1] - a[:, 1]).max() / np.abs(a[:, 1]).max())}
    res["seconds"] = time.perf_counter() - t0
    return res


def run_adjoint(args):
    """Adjoint configuration: dS_z(t_f)/d(6 per-mode coupling scales, impurity scale) on the Si-like
    nk = 500 system (e-ph + e-imp operators kept per mode), RK4 dt = 1 fs, checkpoints every 200
    steps; timed against the forward alone and checked against central differences (h = 1e-4)."""
    import dataclasses
    from denmat_dynm_development_gb300 import host as H
    from denmat_dynm_development_gb300.adjoint import ModeScaledRK4
    name = args.workload if args.workload in ("si_nk500", "mos2_nk2k") else "si_nk500"
    cfg = dataclasses.replace(S.WORKLOADS[name], eimp_sigma_mev=5.0)
    st, P1m, P2m, Q1, Q2 = S.mode_operators(cfg)
    P1m = np.concatenate([P1m, Q1[None]])
    P2m = np.concatenate([P2m, Q2[None]])
    e = np.ascontiguousarray(st.e)
    f = H.fermi(st.T, st.mu, e)
    dm0 = H.dm_bpert(st.s, e, f, st.T, np.array([0.0, 0.0, 0.1 * U.Tesla2au]), 0.0, 0)
    nk_full = float(st.n) ** 3
    ob_prefac = (1.0 / nk_full) / (st.V * U.bohr2cm ** 3)
    nb = cfg.nb
    dt = 1.0 * U.fs
    nsteps = int(round(args.adj_tf_ps * 1000.0))
    theta = np.array([1.0] * cfg.nmodes + [0.2])
    model = ModeScaledRK4(nk=cfg.nk, nb_dm=nb, bstart=0, bend=nb, e_dm=e, k1st=st.k1, k2nd=st.k2, P1_modes=P1m,
                          P2_modes=P2m, prefac_eph=2 * math.pi / nk_full,
                          y0=np.ascontiguousarray(dm0).view(np.float64).reshape(-1), dt=dt, nsteps=nsteps,
                          obs_steps=[nsteps], obs=np.ascontiguousarray(st.s[:, 2, :]), f_obs=f, ob_prefac=ob_prefac,
                          obs_bstart=0, picture=0, expt=1, precision="f64x", checkpoint=200)
    model.forward(theta)  # warm-up (library load, first launches)
    t0 = time.perf_counter()
    s_f = model.forward(theta)[-1]
    fwd_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    s_a, grad = model.gradient(theta, [1.0])
    adj_s = time.perf_counter() - t0
    fd = []
    for m in range(theta.size):
        ep = np.zeros(theta.size)
        ep[m] = 1e-4 * theta[m]
        fd.append((model.forward(theta + ep)[-1] - model.forward(theta - ep)[-1]) / (2e-4 * theta[m]))
    fd = np.array(fd)
    err = np.abs(grad - fd) / np.abs(fd)
    line = {"metric": "adjoint: dS_z(t_f)/d(6 mode scales, n_imp scale), t_f = %g ps" % args.adj_tf_ps,
            "value": adj_s, "unit": "s (forward with checkpoints + backward, 7 gradients)", "n_gpus": 1,
            "higher_is_better": False, "vs_baseline": None, "dtype": "f64 (fp32-pair emulated forward sums)",
            "data": "synthetic", "forward_s": fwd_s, "adjoint_over_forward": adj_s / fwd_s,
            "rk4_steps": nsteps, "s_z_tf": s_f, "s_z_tf_adjoint_pass": s_a[-1], "grad": grad.tolist(),
            "fd_central_h1e-4": fd.tolist(), "rel_err_vs_fd": err.tolist(), "max_rel_err_vs_fd": float(err.max()),
            "config": {"workload": "%s + e-imp (sigma 5 meV): nb=%d, nk=%d, %d k-pairs, %d modes kept apart + "
                                   "impurity operator, theta = (1,..,1, 0.2), Bz_pert 0.1 T, RK4 dt=1 fs, "
                                   "checkpoint every 200 steps" % (name, nb, cfg.nk, st.npair, cfg.nmodes)}}
    print(json.dumps(line))


def run_adjoint_streamed(args):
    """Adjoint configuration at full size on the MoS2-like system (nb = 4, nk = 30k, 4.19M pairs,
    e-ph + e-imp): dS_z(t_f)/d(6 mode scales, impurity scale) through StreamedModeScaledRK4 -- the
    operator sets (34 GB each in complex128) are regenerated chunk by chunk and never held together,
    dJ/dP stays in one shared-memory buffer, and the central differences (h = 1e-4) shift one set in
    place on the device."""
    import dataclasses
    from denmat_dynm_development_gb300 import host as H
    from denmat_dynm_development_gb300.adjoint import StreamedModeScaledRK4
    name = args.workload
    cfg = dataclasses.replace(S.WORKLOADS[name], eimp_sigma_mev=5.0)
    t_start = time.perf_counter()
    ms = S.ModeSets(cfg, procs=max(1, min(16, os.cpu_count() or 1)))
    st = ms.st
    e = np.ascontiguousarray(st.e)
    f = H.fermi(st.T, st.mu, e)
    dm0 = H.dm_bpert(st.s, e, f, st.T, np.array([0.0, 0.0, 0.1 * U.Tesla2au]), 0.0, 0)
    nk_full = float(st.n) ** 3
    nb = cfg.nb
    dt = 1.0 * U.fs
    nsteps = int(round(args.adj_tf_ps * 1000.0))
    theta = np.array([1.0] * cfg.nmodes + [0.2])
    model = StreamedModeScaledRK4(modes=ms, nk=cfg.nk, nb_dm=nb, bstart=0, bend=nb, e_dm=e, k1st=st.k1, k2nd=st.k2,
                                  prefac_eph=2 * math.pi / nk_full, y0=np.ascontiguousarray(dm0).view(np.float64).reshape(-1),
                                  dt=dt, nsteps=nsteps, obs_steps=[nsteps], obs=np.ascontiguousarray(st.s[:, 2, :]), f_obs=f,
                                  ob_prefac=(1.0 / nk_full) / (st.V * U.bohr2cm ** 3), theta=theta, picture=0, expt=1,
                                  precision=args.adj_precision, checkpoint=200)
    setup_s = time.perf_counter() - t_start
    try:
        model.forward()  # warm-up
        t0 = time.perf_counter()
        s_f = model.forward()[-1]
        fwd_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        s_a, grad = model.gradient([1.0])
        adj_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        fd = model.central_differences([1.0], 1e-4)
        fd_s = time.perf_counter() - t0
        pbytes = model.g.pair_bytes
    finally:
        model.close()
    err = np.abs(grad - fd) / np.abs(fd)
    line = {"metric": "adjoint at full size: dS_z(t_f)/d(6 mode scales, n_imp scale), t_f = %g ps" % args.adj_tf_ps,
            "value": adj_s, "unit": "s (forward with checkpoints + backward + per-mode contraction, 7 gradients)",
            "n_gpus": 1, "higher_is_better": False, "vs_baseline": None,
            "dtype": {"f64": "f64", "f64x": "f64 (fp32-pair emulated forward sums)"}[args.adj_precision] +
                     "; backward and dJ/dP in FP64",
            "data": "synthetic", "forward_s": fwd_s, "adjoint_over_forward": adj_s / fwd_s, "rk4_steps": nsteps,
            "setup_s": setup_s, "central_differences_s": fd_s, "gradient_split": getattr(model, "last_timing", None),
            "s_z_tf": s_f, "s_z_tf_adjoint_pass": float(s_a[-1]),
            "grad": grad.tolist(), "fd_central_h1e-4": fd.tolist(), "rel_err_vs_fd": err.tolist(),
            "max_rel_err_vs_fd": float(err.max()),
            "config": {"workload": "%s + e-imp (sigma 5 meV): nb=%d, nk=%d, %d k-pairs (one operator set %.1f GB "
                                   "complex128; 7 sets regenerated chunk by chunk), theta = (1,..,1, 0.2), Bz_pert "
                                   "0.1 T, RK4 dt=1 fs, checkpoint every 200 steps, device operator store %.1f GB"
                                   % (name, nb, cfg.nk, st.npair, 2 * st.npair * nb ** 4 * 16 / 1e9, pbytes / 1e9)}}
    print(json.dumps(line))


def run_temperatures(args):
    """Batched form over separate P sets: 8 temperatures 50-400 K on GaAs-like systems of uneven nk
    (5k-20k), each a tensor-core batch of states (bf16 hi+lo), advanced together by dmd_group_rk4
    (one CUDA graph launch per RK4 step, one parallel branch per temperature)."""
    import dataclasses
    from denmat_dynm_development_gb300.dmd import Group, LindbladGPU
    temps = np.linspace(50.0, 400.0, 8)
    nks = np.linspace(5000, 20000, 8).astype(int)
    R = args.nrhs if args.nrhs > 1 else 12
    h = 1.0 * U.fs
    hs, pairs, desc = [], 0, []
    t0 = time.time()
    for i, (T, nk) in enumerate(zip(temps, nks)):
        cfg = dataclasses.replace(S.WORKLOADS["gaas_nk20k"], nk=int(nk), temperature_K=float(T), seed=100 + i)
        w = build_workload("gaas_nk20k", max(1, min(16, os.cpu_count() or 1)), cfg)
        st = w["st"]
        g = LindbladGPU(nk=st.cfg.nk, nb_dm=st.cfg.nb, bstart=0, bend=st.cfg.nb, e_dm=w["e"], k1st=st.k1, k2nd=st.k2,
                        P1=w["P1"], P2=w["P2"], prefac_eph=w["prefac"], picture=0, expt=1, precision="bf16x2",
                        f_ref=w["f"], nrhs=R)
        g.set_state(0.0, batch_states(w, R, seed=7 + i))
        hs.append(g)
        pairs += st.npair
        desc.append("%gK/nk%d/%dpairs" % (T, nk, st.npair))
        del w
    setup_s = time.time() - t0
    # each system alone, one after another
    for g in hs:
        g.rk4(h, args.warmup)
    t0 = time.perf_counter()
    for g in hs:
        g.rk4(h, args.steps)
    alone_s = time.perf_counter() - t0
    with Group(hs) as grp:
        grp.rk4(h, args.warmup)
        clk = ClockSampler(0)
        clk.start()
        t0 = time.perf_counter()
        grp.rk4(h, args.steps)
        grp_s = time.perf_counter() - t0
        clocks = clk.stop()
    launches = sum(g.launches for g in hs)
    for g in hs:
        g.close()
    nstates = R * len(hs)
    line = {"metric": "ensemble RK4 steps/s over 8 temperatures (separate P sets, %d states each), one graph per step"
                      % R, "value": nstates * args.steps / grp_s, "unit": "state-steps/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": grp_s * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16x2 (rho as deviation from f)",
            "data": "synthetic", "sequential_state_steps_per_s": nstates * args.steps / alone_s,
            "group_speedup_over_sequential": alone_s / grp_s,
            "config": {"workload": "8 GaAs-like P sets: " + ", ".join(desc), "total_pairs": pairs, "states": nstates,
                       "setup_s": setup_s, "timing": "host wall clock around the synchronised group launches"},
            "clocks": clocks, "gpu_launches_total": launches}
    print(json.dumps(line))


def ee_survivors(st, kidx, table, n, ethr, pairs):
    """(k1, k2, k3) with k4 = k1 + k3 - k2 on the k-point set and some band combination inside the
    energy window (the reference's calc_P work items), counted for the given pairs"""
    ew = st.ew
    nk = ew.shape[0]
    cnt = 0
    for p in pairs:
        k1, k2 = int(st.k1[p]), int(st.k2[p])
        m = (kidx[k1][None, :] + kidx - kidx[k2][None, :]) % n
        k4 = table[m[:, 0], m[:, 1], m[:, 2]]
        ok = k4 >= 0
        k3 = np.nonzero(ok)[0]
        k4 = k4[ok]
        de = (ew[k1][:, None, None, None] - ew[k2][None, :, None, None])[None] + \
             (ew[k3][:, None, :, None] - ew[k4][:, None, None, :])[:, None]
        cnt += int(np.any(np.abs(de.reshape(k3.size, -1)) < ethr, axis=1).sum())
    return cnt


def run_ee(args):
    """e-e operators rebuilt from rho (eeMode = Pee_update, Debye screening updated from rho): the
    rebuild alone (P_ee of every pair from the state, refill of the stored operators) and RK4 with the
    rebuild before every RHS evaluation, on a ball of k-points of a GaAs-like mesh."""
    from denmat_dynm_development_gb300 import host as H
    from denmat_dynm_development_gb300.dmd import LindbladGPU
    nb = args.ee_nb
    nbw = 2 * nb
    cfg = S.SynthConfig(nk=args.ee_nk, nb=nb, seed=51, de_pair_mev=args.ee_de_mev, nwannier=nbw, kball=True)
    t0 = time.time()
    st, P1, P2, _, _ = S.generate_arrays(cfg, procs=max(1, min(16, os.cpu_count() or 1)))
    gen_s = time.time() - t0
    T, mu = st.T, st.mu
    e = np.ascontiguousarray(st.e)
    f = H.fermi(T, mu, e)
    dm0 = H.dm_bpert(st.s, e, f, T, np.array([0.0, 0.0, 0.1 * U.Tesla2au]), 0.0, 0)
    nk_full, V, n = float(st.n) ** 3, st.V, st.n
    G = 2.0 * math.pi * np.linalg.inv(st.R)
    degauss = cfg.degauss_mev * 1e-3 * U.eV
    ee = dict(kvec=st.kf, kmesh=(n, n, n), U=S.umat(cfg, st.kf)[:, :, :nb], f=f, GGT=G @ G.T, cell_size=V,
              nk_full=nk_full, temperature=T, eps_background=12.9, meff=0.3, formula="debye",
              nfree=float(f.sum()) / (nk_full * V), update_screening=1, nv=0, degauss=degauss,
              ethr=degauss * cfg.ndegauss, antisymmetry=0, scale=1.0, every_rhs=1)
    prec = args.precision
    g = LindbladGPU(nk=cfg.nk, nb_dm=nb, bstart=0, bend=nb, e_dm=e, k1st=st.k1, k2nd=st.k2, P1=P1, P2=P2,
                    prefac_eph=2 * math.pi / nk_full, picture=0, expt=1, precision=prec, ee=ee)
    y0 = np.ascontiguousarray(dm0).view(np.float64).reshape(-1)
    g.set_state(0.0, y0)
    for _ in range(args.warmup):
        g.ee_update()
    clk = ClockSampler(0)
    clk.start()
    g.sync()
    l0 = g.launches
    g.timer_start()
    for _ in range(args.steps):
        g.ee_update()
    ms = g.timer_stop() / args.steps
    clocks = clk.stop()
    launches = g.launches - l0
    g.set_profiling(True)
    g.ee_update()
    g.set_profiling(False)  # harvests the recorded events
    reb_ms, reb_n = g.profile(4)
    # RK4 with the rebuild before every stage (freq_update_ee_model < 0)
    h = 1.0 * U.fs
    nst = max(3, args.steps // 4)
    g.rk4(h, args.warmup)
    g.sync()
    g.timer_start()
    g.rk4(h, nst)
    rk_ms = g.timer_stop() / nst
    g.close()
    # work items of the reference's loop (exact count on a pair sample, scaled), flops per item
    kidx = np.rint(n * (st.kf - np.floor(st.kf))).astype(np.int64) % n
    table = -np.ones((n, n, n), np.int64)
    for k in range(cfg.nk - 1, -1, -1):
        table[tuple(kidx[k])] = k
    rng = np.random.default_rng(3)
    sample = rng.choice(st.npair, size=min(st.npair, 400), replace=False)
    surv = ee_survivors(st, kidx, table, n, ee["ethr"], sample) * st.npair / sample.size
    flops_item = 8 * (nb * nb * nbw + 4 * nb ** 5 + 2 * nb ** 6) + 8 * nb ** 4
    flops = surv * flops_item
    peak = 1250.0
    line = {"metric": "e-e operator rebuilds/s (P_ee of every k-pair from rho, Pee_update)", "value": 1e3 / ms,
            "unit": "rebuilds/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "ee_ball_nk%d: nb=%d, nk=%d (ball of a %d^3 mesh), %d k-pairs, %d Wannier functions, "
                                   "Debye screening from rho, Lindblad e-e (ElecElec_Model.h:186-262)"
                                   % (cfg.nk, nb, cfg.nk, n, st.npair, nbw),
                       "npair": st.npair, "nk": cfg.nk, "k3_candidates": st.npair * cfg.nk,
                       "work_items_estimated": surv, "work_item_sample_pairs": int(sample.size),
                       "l2": "per rebuild the operators (%.2f GB) are read and written; no flush" %
                             (2 * st.npair * nb ** 4 * 16 * 2 / 1e9),
                       "gen_s": gen_s},
            "rk4_with_every_rhs_rebuild": {"steps_per_s": 1e3 / rk_ms, "ms_per_step": rk_ms, "precision": prec},
            "roofline": {"bound": "fp64", "achieved": flops / (ms * 1e-3) / 1e9, "peak": peak, "unit": "GFLOP/s",
                         "frac": flops / (ms * 1e-3) / 1e9 / peak, "traffic": None, "peak_kind": "nominal FP64",
                         "kernel": "e-e rebuild (k_ee_pairs + refill)", "flops_per_work_item": flops_item,
                         "profiled_rebuild_ms": reb_ms / max(reb_n, 1)},
            "clocks": clocks, "gpu_launches": launches}
    if args.cpu_baseline:
        line["cpu_baseline"] = ee_cpu_baseline(st, P1, P2, e, f, ee, nb)
    print(json.dumps(line))


def ee_cpu_baseline(st, P1, P2, e, f, ee, nb):
    """the oracle's calc_P restatement (one core) on a bounded sample of the pairs"""
    from oracle import oracle as O
    O.build()

    order = np.random.default_rng(7).permutation(st.npair)

    def timed(m):
        idx = np.sort(order[:m])  # a random sample: the pairs' work varies along the stored order
        s = O.from_arrays(nk=st.cfg.nk, nb_dm=nb, bstart=0, bend=nb, e_dm=e, f_dm=f, k1st=st.k1[idx], k2nd=st.k2[idx],
                          P1=P1[idx], P2=P2[idx], prefac_eph=1.0, dm0=np.zeros((st.cfg.nk, nb * nb), np.complex128))
        m_ = O.EEModel(nb=nb, kvec=ee["kvec"], kmesh=ee["kmesh"], U=ee["U"], GGT=ee["GGT"], cell_size=ee["cell_size"],
                       nk_full=ee["nk_full"], T=ee["temperature"], eps=ee["eps_background"], meff=ee["meff"],
                       formula=ee["formula"], nfree=ee["nfree"], update_screening=1, nv=0, degauss=ee["degauss"],
                       ethr=ee["ethr"], antisym=0, scale=1.0, inside=0, P1base=P1[idx].reshape(-1),
                       P2base=P2[idx].reshape(-1))
        dmw = np.zeros((st.cfg.nk, nb * nb), np.complex128)
        dmw[:, 0], dmw[:, 3] = f[:, 0], f[:, 1]
        t0 = time.perf_counter()
        O.ee_operators(s, m_, dmw, None, ee["nfree"])
        return time.perf_counter() - t0

    m = 50
    dt = timed(m)
    m2 = int(min(st.npair, max(m, m * 15.0 / max(dt, 1e-3))))
    dt2 = timed(m2) if m2 > m else dt
    pairs_s = m2 / dt2
    return {"value": pairs_s / st.npair, "unit": "rebuilds/s", "cores": 1, "kind": "port",
            "sample": "oracle calc_P restatement over %d random pairs of %d (all k3), %.1f s; scaled to a full "
                      "rebuild" % (m2, st.npair, dt2)}


def run_sparse(args):
    """Sparse contraction (alg_sparseP) against the dense FP64 contraction on an nb = 4 MoS2-like P
    with a fraction of each pair's elements kept at random (the rest set to zero): per fill, the
    event-timed contraction launch of both forms on the same operators, RK4 steps/s, and the sparse
    form's RHS against the dense form's."""
    import dataclasses
    nk = args.sparse_nk
    cfg = dataclasses.replace(S.WORKLOADS["mos2_nk30k"], nk=nk)
    w = build_workload("mos2_nk30k", max(1, min(16, os.cpu_count() or 1)), cfg)
    st = w["st"]
    nb = st.cfg.nb
    h = 1.0 * U.fs
    y0 = np.ascontiguousarray(w["dm0"]).view(np.float64).reshape(-1).copy()
    P1d, P2d = w["P1"], w["P2"]
    rng = np.random.default_rng(77)
    u = rng.random(P1d.shape)  # one draw per element: fills are nested
    dense_bytes = 2 * st.npair * nb ** 4 * 16
    rows = []
    from denmat_dynm_development_gb300.dmd import LindbladGPU
    for fill in [float(x) for x in args.sparse_fills.split(",")]:
        keep = u < fill
        P1 = np.where(keep, P1d, 0)
        P2 = np.where(keep, P2d, 0)
        r = {"fill": fill, "stored_fraction": float(np.mean((P1 != 0) | (P2 != 0)))}
        out = {}
        for form in ("dense", "sparse"):
            g = LindbladGPU(nk=st.cfg.nk, nb_dm=nb, bstart=0, bend=nb, e_dm=w["e"], k1st=st.k1, k2nd=st.k2, P1=P1,
                            P2=P2, prefac_eph=w["prefac"], picture=0, expt=1, precision="f64",
                            sparse=(form == "sparse"))
            try:
                g.set_state(0.0, y0)
                out[form] = g.func(3.0 * U.fs, y0)
                g.rk4(h, args.warmup)
                tm = Timed(g, h, args.steps, 3)
                kms, _ = kernel_profile(g, h, max(2, min(args.steps, 10)))
                r[form] = {"rk4_steps_per_s": 1e3 * args.steps / tm.median, "contraction_ms": kms["pairs"],
                           "stored_bytes": g.pair_bytes}
            finally:
                g.close()
        r["speedup"] = r["dense"]["contraction_ms"] / r["sparse"]["contraction_ms"]
        r["sparse_vs_dense_rhs_rel_err"] = rel_err(out["sparse"], out["dense"])
        r["faster"] = "sparse" if r["speedup"] > 1.0 else "dense"
        rows.append(r)
    mid = rows[len(rows) // 2]
    line = {"metric": "sparse vs dense FP64 k-pair contraction (alg_sparseP), nb = 4", "value": mid["speedup"],
            "unit": "x (dense / sparse contraction time at fill %.2f)" % mid["fill"], "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "mos2-like nb=4, nk=%d, %d k-pairs (dense P1+P2 %.2f GB complex128); each element "
                                   "kept with probability = fill, the rest zero" % (nk, st.npair, dense_bytes / 1e9)},
            "fills": rows}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="gaas_nk20k")
    ap.add_argument("--precision", default="f64", choices=["f64", "f64x", "f32", "bf16x2"])
    ap.add_argument("--windows", type=int, default=5, help="timed K-step windows (median reported)")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="keep the default contraction shape (profiling runs)")
    ap.add_argument("--no-forms", dest="forms", action="store_false",
                    help="skip the other arithmetics of the contraction")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-t1", dest="t1", action="store_false")
    ap.add_argument("--t1-steps", type=int, default=10000)
    ap.add_argument("--nrhs", type=int, default=1, help="batched form: states sharing P (f32 / bf16x2)")
    ap.add_argument("--adjoint", action="store_true", help="adjoint configuration (gradients of S_z(t_f))")
    ap.add_argument("--temperatures", action="store_true", help="batched form over 8 temperature P sets")
    ap.add_argument("--adj-tf-ps", type=float, default=50.0, help="adjoint: t_f in ps")
    ap.add_argument("--adj-precision", default="f64x", choices=["f64", "f64x"],
                    help="adjoint at full size: arithmetic of the forward sums")
    ap.add_argument("--ee", action="store_true", help="e-e operators rebuilt from rho (Pee_update)")
    ap.add_argument("--sparse", action="store_true", help="sparse vs dense FP64 contraction at several fills")
    ap.add_argument("--sparse-nk", type=int, default=12000, help="sparse: k-points of the nb = 4 system")
    ap.add_argument("--sparse-fills", default="0.1,0.2,0.35,0.5", help="sparse: kept fractions of the elements")
    ap.add_argument("--ee-nk", type=int, default=2000, help="e-e: k-points of the ball")
    ap.add_argument("--ee-de-mev", type=float, default=20.0, help="e-e: pair energy window (meV)")
    ap.add_argument("--ee-nb", type=int, default=2, choices=[2, 4], help="e-e: bands of the window")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world = env_int("RANK", 0), env_int("WORLD_SIZE", 1)
    if args.impl == "reference":
        if rank != 0:
            return
        w = build_workload(args.workload, min(16, os.cpu_count() or 1), setup="oracle")
        run_reference(args, w)
        return
    if args.adjoint:
        if rank == 0:
            if args.workload == "mos2_nk30k":  # full size: operator sets streamed
                run_adjoint_streamed(args)
            else:
                run_adjoint(args)
        return
    if args.temperatures:
        if rank == 0:
            run_temperatures(args)
        return
    if args.ee:
        if rank == 0:
            run_ee(args)
        return
    if args.sparse:
        if rank == 0:
            run_sparse(args)
        return
    # the generator's worker processes start before any CUDA call
    w = build_workload(args.workload, max(1, min(16, (os.cpu_count() or 1) // max(world, 1))))
    if args.nrhs > 1:
        if rank == 0:
            run_gpu_batched(args, w)
        return
    dist = None
    if world > 1:
        import torch
        import torch.distributed as D
        torch.cuda.set_device(env_int("LOCAL_RANK", 0))
        D.init_process_group("nccl")
        dist = D
    try:
        run_gpu(args, w, rank, world, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
