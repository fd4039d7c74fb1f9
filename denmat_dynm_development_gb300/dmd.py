"""Python binding of the GPU C ABI (include/dmd_gpu.h) through ctypes.

``LindbladGPU`` mirrors the reference's call surface for this path: ``func`` is the GSL callback
of DensityMatrix_Dynamics.h:358-369, ``evolve_driver`` is electronphonon::evolve_driver
(evolve_eph.cpp:21-32), ``evolve_coh`` is singdenmat_k::evolve_coh (DenMat.cpp:29-55); the
steppers run with the density matrix resident on the GPU. There is no CPU fallback: without the
compiled library or a CUDA device every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from .build import GPU_LIB

PREC = {"f64": 0, "f64x": 1, "f32": 2, "bf16x2": 3}
FLAG_LINEAR = 1  # DMD_FLAG_LINEAR: P1, P2 are the linear operators Lscij, Lscji
FLAG_ADJOINT = 2  # DMD_FLAG_ADJOINT: keep the operators in stored order for adjoint_rk4
FLAG_EE = 4  # DMD_FLAG_EE: keep P_eph (+ P_eimp) in stored order and the column-block map for the e-e model
FLAG_SPARSE = 8  # DMD_FLAG_SPARSE: contract only the stored elements (alg_sparseP / alg_Pin_is_sparse)
# sparse="auto" picks the sparse FP64 contraction below this fraction of stored elements: on an nb = 4
# MoS2-like workload (727k pairs) it ran 4.7x / 2.5x / 1.45x / 1.02x faster than the dense FP64
# contraction at 9 / 18 / 31 / 44 % stored (bench --sparse)
SPARSE_AUTO_FILL = 0.4


def stored_fraction(P1, P2, thr=1e-40):
    """fraction of the elements of P1, P2 with |P| > thr (what the sparse form keeps)"""
    n = 0
    for P in (P1, P2):
        n += int(np.count_nonzero(np.abs(np.asarray(P)) > thr))
    return n / max(1, np.asarray(P1).size + np.asarray(P2).size)
PICTURE = {"interaction": 0, "schrodinger": 1}


class DMDError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("dmd status %d (%s): %s" % (status, _lib().dmd_strerror(status).decode(), msg))
        self.status = status


class _Desc(C.Structure):
    _fields_ = [("nk", C.c_int32), ("nb_dm", C.c_int32), ("bstart", C.c_int32), ("bend", C.c_int32),
                ("nkpair", C.c_int64), ("prefac_eph", C.c_double), ("e_dm", C.c_void_p), ("k1st", C.c_void_p),
                ("k2nd", C.c_void_p), ("P1", C.c_void_p), ("P2", C.c_void_p), ("P1_add", C.c_void_p),
                ("P2_add", C.c_void_p), ("add_scale", C.c_double), ("Hcoh", C.c_void_p), ("picture", C.c_int32),
                ("expt", C.c_int32), ("precision", C.c_int32), ("device", C.c_int32), ("flags", C.c_uint32),
                ("f_ref", C.c_void_p), ("nrhs", C.c_int32), ("reserved", C.c_int32)]


class _EEDesc(C.Structure):
    """dmd_ee_desc (include/dmd_gpu.h)"""
    _fields_ = [("nbw", C.c_int32), ("kvec", C.c_void_p), ("kmesh", C.c_int32 * 3), ("U", C.c_void_p),
                ("f", C.c_void_p), ("GGT", C.c_double * 9), ("cell_size", C.c_double), ("nk_full", C.c_double),
                ("temperature", C.c_double), ("eps_background", C.c_double), ("meff", C.c_double),
                ("formula", C.c_int32), ("nfree", C.c_double), ("update_screening", C.c_int32), ("nv", C.c_int32),
                ("degauss", C.c_double), ("ethr", C.c_double), ("antisymmetry", C.c_int32), ("scale", C.c_double),
                ("every_rhs", C.c_int32), ("dynamic", C.c_int32), ("ppa_gn", C.c_int32), ("eppa", C.c_double),
                ("smearing", C.c_double), ("two_freqs", C.c_int32)]


SCREEN = {"unscreened": 0, "debye": 1, "Bechstedt": 2, "RPA": 3}

_L = None

EXPORTS = ["dmd_create", "dmd_destroy", "dmd_last_error", "dmd_strerror", "dmd_set_ddmdt_eq", "dmd_func",
           "dmd_evolve_driver", "dmd_evolve_coh", "dmd_set_state", "dmd_get_state", "dmd_rk4", "dmd_euler",
           "dmd_rkf45_apply", "dmd_set_observable", "dmd_measure", "dmd_launch_count", "dmd_sync",
           "dmd_pinned_alloc", "dmd_pinned_free", "dmd_timer", "dmd_set_profiling", "dmd_profile_get",
           "dmd_evolve_driver_noalloc", "dmd_measure_batch", "dmd_pair_bytes", "dmd_adjoint_rk4", "dmd_autotune",
           "dmd_group_create", "dmd_group_rk4", "dmd_group_destroy",
           "dmd_create_from_files", "dmd_create_from_sparse_files", "dmd_selftest_wait_timeout", "dmd_peak_fma", "dmd_add_operators", "dmd_ee_linear_terms",
           "dmd_ee_attach", "dmd_ee_update", "dmd_ee_read"]


def _lib():
    global _L
    if _L is None:
        if not os.path.exists(GPU_LIB):
            raise RuntimeError("libdmdgpu.so is not built (call __graft_entry__.build() or "
                               "denmat_dynm_development_gb300.build.build_all())")
        L = C.CDLL(GPU_LIB)
        vp, d, i64 = C.c_void_p, C.c_double, C.c_int64
        L.dmd_create.argtypes = [C.POINTER(_Desc), C.POINTER(vp)]
        L.dmd_destroy.argtypes = [vp]
        L.dmd_last_error.argtypes = [vp]
        L.dmd_last_error.restype = C.c_char_p
        L.dmd_strerror.argtypes = [C.c_int]
        L.dmd_strerror.restype = C.c_char_p
        L.dmd_set_ddmdt_eq.argtypes = [vp, vp]
        L.dmd_func.argtypes = [vp, d, vp, vp]
        L.dmd_evolve_driver.argtypes = [vp, d, vp, vp, vp]
        L.dmd_evolve_coh.argtypes = [vp, d, vp, vp]
        L.dmd_set_state.argtypes = [vp, d, vp]
        L.dmd_get_state.argtypes = [vp, C.POINTER(d), vp]
        L.dmd_rk4.argtypes = [vp, d, i64]
        L.dmd_euler.argtypes = [vp, d, i64]
        L.dmd_rkf45_apply.argtypes = [vp, d, C.POINTER(d), d, d, d, d, C.POINTER(i64)]
        L.dmd_set_observable.argtypes = [vp, C.c_int, vp, vp, d]
        L.dmd_measure_batch.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, vp]
        L.dmd_measure.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(d), C.POINTER(d)]
        L.dmd_launch_count.argtypes = [vp, C.POINTER(i64)]
        L.dmd_pair_bytes.argtypes = [vp, C.POINTER(i64)]
        L.dmd_autotune.argtypes = [vp, C.c_int, C.POINTER(C.c_int)]
        L.dmd_group_create.argtypes = [C.POINTER(vp), C.c_int, C.POINTER(vp)]
        L.dmd_group_rk4.argtypes = [vp, d, i64]
        L.dmd_group_destroy.argtypes = [vp]
        L.dmd_selftest_wait_timeout.argtypes = [C.c_int, C.c_uint32, C.POINTER(C.c_int)]
        L.dmd_peak_fma.argtypes = [C.c_int, C.c_int, C.POINTER(d)]
        L.dmd_add_operators.argtypes = [vp, vp, vp, d]
        L.dmd_ee_linear_terms.argtypes = [vp, vp, d, vp, vp, vp, vp, vp, vp]
        L.dmd_create_from_files.argtypes = [C.POINTER(_Desc), C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p,
                                            C.POINTER(vp)]
        L.dmd_create_from_sparse_files.argtypes = [C.POINTER(_Desc), C.c_char_p, C.c_char_p, C.c_char_p,
                                                   C.c_char_p, C.POINTER(vp)]
        L.dmd_adjoint_rk4.argtypes = [vp, d, vp, d, i64, i64, C.c_int, C.c_int, C.c_int, i64, vp, vp, vp, vp, vp]
        L.dmd_ee_attach.argtypes = [vp, C.POINTER(_EEDesc)]
        L.dmd_ee_update.argtypes = [vp]
        L.dmd_ee_read.argtypes = [vp, vp, vp, C.POINTER(d)]
        L.dmd_sync.argtypes = [vp]
        L.dmd_pinned_alloc.argtypes = [C.c_size_t, C.POINTER(vp)]
        L.dmd_pinned_free.argtypes = [vp]
        L.dmd_timer.argtypes = [vp, C.c_int, C.POINTER(d)]
        L.dmd_set_profiling.argtypes = [vp, C.c_int]
        L.dmd_profile_get.argtypes = [vp, C.c_int, C.POINTER(d), C.POINTER(i64)]
        L.dmd_evolve_driver_noalloc.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, i64, vp, vp, vp, vp, vp, d,
                                                C.c_int32, d, vp, vp, vp]
        _L = L
    return _L


def peak_fma(device: int = 0, fp64: bool = True) -> float:
    """Measured fused multiply-add throughput of the device in TFLOP/s (dmd_peak_fma)."""
    v = C.c_double(0.0)
    st = _lib().dmd_peak_fma(int(device), 1 if fp64 else 0, C.byref(v))
    if st != 0:
        raise DMDError(st, "dmd_peak_fma failed")
    return float(v.value)


def _c(a, dtype):
    return None if a is None else np.ascontiguousarray(a, dtype=dtype)


class LindbladGPU:
    """Device-resident Lindblad RHS for one set of k-pair operators."""

    def __init__(self, *, nk, nb_dm, bstart, bend, e_dm, k1st, k2nd, P1, P2, prefac_eph, Hcoh=None,
                 picture="interaction", expt=1, precision="f64", P1_add=None, P2_add=None, add_scale=0.0, device=0,
                 f_ref=None, linear=False, nrhs=1, adjoint=False, P_files=None, P_sparse=None, ee=None,
                 ee_flag=False, sparse=False):
        L = _lib()
        self._keep = dict(e=_c(e_dm, np.float64), k1=_c(k1st, np.uint64), k2=_c(k2nd, np.uint64),
                          P1=_c(P1, np.complex128), P2=_c(P2, np.complex128), H=_c(Hcoh, np.complex128),
                          A1=_c(P1_add, np.complex128), A2=_c(P2_add, np.complex128), f=_c(f_ref, np.float64))
        k = self._keep
        if sparse == "auto":  # the faster form for the operators' fill (dense P given as arrays)
            sparse = (precision in ("f64", 0) and nrhs <= 1 and not (linear or adjoint or ee or ee_flag) and
                      k["P1"] is not None and k["A1"] is None and
                      stored_fraction(k["P1"], k["P2"]) < SPARSE_AUTO_FILL)
        ptr = lambda a: None if a is None else a.ctypes.data  # noqa: E731
        desc = _Desc(nk=nk, nb_dm=nb_dm, bstart=bstart, bend=bend, nkpair=int(k["k1"].size), prefac_eph=prefac_eph,
                     e_dm=ptr(k["e"]), k1st=ptr(k["k1"]), k2nd=ptr(k["k2"]), P1=ptr(k["P1"]), P2=ptr(k["P2"]),
                     P1_add=ptr(k["A1"]), P2_add=ptr(k["A2"]), add_scale=add_scale, Hcoh=ptr(k["H"]),
                     picture=PICTURE[picture] if isinstance(picture, str) else int(picture), expt=int(expt),
                     precision=PREC[precision] if isinstance(precision, str) else int(precision), device=device,
                     flags=(FLAG_LINEAR if linear else 0) | (FLAG_ADJOINT if adjoint else 0) |
                     (FLAG_EE if (ee or ee_flag) else 0) | (FLAG_SPARSE if sparse else 0),
                     f_ref=ptr(k["f"]),
                     nrhs=int(nrhs))
        h = C.c_void_p()
        if P_files is not None:  # DMD's operator files, streamed by the library
            fp = [None if f is None else os.fsencode(f) for f in (list(P_files) + [None, None])[:4]]
            st = L.dmd_create_from_files(C.byref(desc), fp[0], fp[1], fp[2], fp[3], C.byref(h))
        elif P_sparse is not None:  # DMD's sparse operator files (prefixes), plus optional dense additive files
            fp = [None if f is None else os.fsencode(f) for f in (list(P_sparse) + [None, None])[:4]]
            st = L.dmd_create_from_sparse_files(C.byref(desc), fp[0], fp[1], fp[2], fp[3], C.byref(h))
        else:
            st = L.dmd_create(C.byref(desc), C.byref(h))
        if st != 0:
            raise DMDError(st, "dmd_create failed")
        self._h = h
        self._keep = None  # the library copied everything it needs
        self.nk, self.nb_dm, self.nrhs = nk, nb_dm, max(1, int(nrhs))
        self.npair, self.nb4 = int(np.asarray(k1st).size), (bend - bstart) ** 4
        self.ny = 2 * nk * nb_dm * nb_dm * self.nrhs
        if ee:
            try:
                self.ee_attach(**ee)
            except Exception:
                self.close()
                raise

    # ------------------------------------------------------------------ e-e model (eeMode = Pee_update)
    def ee_attach(self, *, kvec, kmesh, U, f, GGT, cell_size, nk_full, temperature, eps_background, meff, formula,
                  nfree, update_screening, nv, degauss, ethr, antisymmetry, scale, every_rhs, dynamic=0, ppa_gn=1,
                  eppa=0.0, smearing=0.0, two_freqs=0):
        """Attach the e-e model (dmd_ee_attach): U complex [nk][nbw][nb], kvec [nk][3] fractional,
        f [nk][nb] window occupations of the set-up, formula "unscreened" / "debye" / "Bechstedt" /
        "RPA"; dynamic = 1 (or "ppa"): plasmon-pole screening (RPA), ppa_gn 1 Godby-Needs / 0
        Hybertsen-Louie, eppa / smearing in Hartree (0: the reference's defaults)."""
        U = np.ascontiguousarray(U, np.complex128)
        keep = dict(kvec=np.ascontiguousarray(kvec, np.float64), U=U, f=np.ascontiguousarray(f, np.float64))
        d = _EEDesc(nbw=int(U.shape[1]), kvec=keep["kvec"].ctypes.data, kmesh=(C.c_int32 * 3)(*[int(x) for x in kmesh]),
                    U=U.ctypes.data, f=keep["f"].ctypes.data,
                    GGT=(C.c_double * 9)(*np.asarray(GGT, np.float64).reshape(9)), cell_size=cell_size,
                    nk_full=nk_full, temperature=temperature, eps_background=eps_background, meff=meff,
                    formula=SCREEN[formula] if isinstance(formula, str) else int(formula), nfree=nfree,
                    update_screening=int(update_screening), nv=int(nv), degauss=degauss, ethr=ethr,
                    antisymmetry=int(antisymmetry), scale=scale, every_rhs=int(every_rhs),
                    dynamic=(1 if dynamic == "ppa" else 0) if isinstance(dynamic, str) else int(dynamic),
                    ppa_gn=(1 if ppa_gn == "gn" else 0) if isinstance(ppa_gn, str) else int(ppa_gn),
                    eppa=float(eppa), smearing=float(smearing), two_freqs=int(two_freqs))
        self._ck(_lib().dmd_ee_attach(self._h, C.byref(d)))

    def ee_update(self):
        """Rebuild P_ee from the handle's state at its time (dmd_ee_update)."""
        self._ck(_lib().dmd_ee_update(self._h))

    def ee_linear_terms(self, f_eq, nfree):
        """P_ee at f_eq and P3..P6 of every pair (the e-e source of the linearized operators):
        complex [6][npair][nb^4], prefactor included, scale_ee not"""
        f = np.ascontiguousarray(f_eq, np.float64)
        out = np.zeros((6, self.npair, self.nb4), np.complex128)
        p = [out[i].ctypes.data for i in range(6)]
        self._ck(_lib().dmd_ee_linear_terms(self._h, f.ctypes.data, float(nfree), *p))
        return out

    def ee_read(self):
        """(P1ee, P2ee complex [npair][nb^4], screening density) of the last rebuild."""
        P1 = np.empty((self.npair, self.nb4), np.complex128)
        P2 = np.empty((self.npair, self.nb4), np.complex128)
        n = C.c_double()
        self._ck(_lib().dmd_ee_read(self._h, P1.ctypes.data, P2.ctypes.data, C.byref(n)))
        return P1, P2, n.value

    # ------------------------------------------------------------------ plumbing
    def _ck(self, st):
        if st != 0:
            raise DMDError(st, _lib().dmd_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            _lib().dmd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _y(self, y):
        y = np.ascontiguousarray(y)
        if y.dtype == np.complex128:
            y = y.view(np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64).reshape(-1)
        if y.size != self.ny:
            raise ValueError("state has %d doubles, expected %d" % (y.size, self.ny))
        return y

    # ------------------------------------------------------------------ reference-facing calls
    def func(self, t, y, dydt=None):
        y = self._y(y)
        out = np.empty_like(y) if dydt is None else dydt
        self._ck(_lib().dmd_func(self._h, float(t), y.ctypes.data, out.ctypes.data))
        return out

    def evolve_driver(self, t, dm, dm1=None):
        y = self._y(dm)
        out = np.empty_like(y)
        self._ck(_lib().dmd_evolve_driver(self._h, float(t), y.ctypes.data, None, out.ctypes.data))
        return out

    def evolve_coh(self, t, dm):
        y = self._y(dm)
        out = np.empty_like(y)
        self._ck(_lib().dmd_evolve_coh(self._h, float(t), y.ctypes.data, out.ctypes.data))
        return out

    def set_ddmdt_eq(self, eq: Optional[np.ndarray]):
        a = None if eq is None else np.ascontiguousarray(eq, dtype=np.complex128)
        self._ck(_lib().dmd_set_ddmdt_eq(self._h, None if a is None else a.ctypes.data))

    # ------------------------------------------------------------------ device-resident stepping
    def set_state(self, t, y):
        y = self._y(y)
        self._ck(_lib().dmd_set_state(self._h, float(t), y.ctypes.data))

    def get_state(self):
        y = np.empty(self.ny, np.float64)
        t = C.c_double()
        self._ck(_lib().dmd_get_state(self._h, C.byref(t), y.ctypes.data))
        return t.value, y

    def rk4(self, dt, nsteps):
        self._ck(_lib().dmd_rk4(self._h, float(dt), int(nsteps)))

    def euler(self, dt, nsteps):
        self._ck(_lib().dmd_euler(self._h, float(dt), int(nsteps)))

    def rkf45_apply(self, t1, hstep, hmin=0.0, hmax=1e300, epsabs=1e-8, epsrel=0.0):
        hs = C.c_double(hstep)
        nf = C.c_int64()
        self._ck(_lib().dmd_rkf45_apply(self._h, float(t1), C.byref(hs), hmin, hmax, epsabs, epsrel, C.byref(nf)))
        return hs.value, nf.value

    def set_observable(self, slot, obs, f, prefac):
        o = np.ascontiguousarray(obs, dtype=np.complex128)
        ff = np.ascontiguousarray(f, dtype=np.float64)
        self._ck(_lib().dmd_set_observable(self._h, slot, o.ctypes.data, ff.ctypes.data, float(prefac)))

    def measure_batch(self, slot=0, bstart=0, bend=None):
        """Totals of every state of a batched handle: arrays (tot, tot_amp) of nrhs values."""
        bend = self.nb_dm if bend is None else bend
        a, b = np.zeros(self.nrhs), np.zeros(self.nrhs)
        self._ck(_lib().dmd_measure_batch(self._h, slot, bstart, bend, a.ctypes.data, b.ctypes.data))
        return a, b

    def measure(self, slot=0, bstart=0, bend=None):
        bend = self.nb_dm if bend is None else bend
        a, b = C.c_double(), C.c_double()
        self._ck(_lib().dmd_measure(self._h, slot, bstart, bend, C.byref(a), C.byref(b)))
        return a.value, b.value

    @property
    def launches(self):
        n = C.c_int64()
        self._ck(_lib().dmd_launch_count(self._h, C.byref(n)))
        return n.value

    def adjoint_rk4(self, t0, y0, dt, nsteps, obs_step, obs_weight, slot=0, bstart=0, bend=None, checkpoint=200,
                    want_dP=True, want_dy0=False, dP_out=None):
        """Reverse mode of `nsteps` RK4 steps from (t0, y0) for J = sum_i w_i S(t0 + obs_step[i] dt) (S: the
        total of observable `slot`). Returns (S at the observed steps, dJ/dP as complex [2][nkpair][nb^4]
        with dJ = Re sum(conj(dJ/dP) dP) or None, dJ/dy0 as y0's layout or None). dP_out: a C-contiguous
        complex128 [2][nkpair][nb^4] array to receive dJ/dP (e.g. in shared memory) instead of a new one."""
        bend = self.nb_dm if bend is None else bend
        y0 = np.ascontiguousarray(y0, dtype=np.float64)
        st = np.ascontiguousarray(obs_step, dtype=np.int64)
        w = np.ascontiguousarray(obs_weight, dtype=np.float64)
        s = np.zeros(st.size)
        if dP_out is not None:
            if dP_out.dtype != np.complex128 or dP_out.size != 2 * self.npair * self.nb4 or not dP_out.flags.c_contiguous:
                raise ValueError("dP_out must be a C-contiguous complex128 [2][nkpair][nb^4] array")
            dP = dP_out.reshape(-1).view(np.float64)
        else:
            dP = np.zeros(2 * self.npair * self.nb4 * 2) if want_dP else None
        dy = np.zeros(self.ny) if want_dy0 else None
        ptr = lambda a: None if a is None else a.ctypes.data  # noqa: E731
        self._ck(_lib().dmd_adjoint_rk4(self._h, float(t0), y0.ctypes.data, float(dt), int(nsteps), int(checkpoint),
                                        int(slot), int(bstart), int(bend), int(st.size), ptr(st), ptr(w), s.ctypes.data,
                                        ptr(dP), ptr(dy)))
        if dP is not None:
            dP = dP.view(np.complex128).reshape(2, self.npair, self.nb4)
        return s, dP, dy

    def add_operators(self, P1_add, P2_add, scale):
        """P += scale * P_add on the device (DMD_FLAG_ADJOINT handles), stored form rebuilt"""
        A1 = np.ascontiguousarray(P1_add, np.complex128)
        A2 = np.ascontiguousarray(P2_add, np.complex128)
        if A1.size != self.npair * self.nb4 or A2.size != self.npair * self.nb4:
            raise ValueError("P1_add, P2_add must hold nkpair * nb^4 elements")
        self._ck(_lib().dmd_add_operators(self._h, A1.ctypes.data, A2.ctypes.data, float(scale)))

    def autotune(self, evals=3):
        """time the compiled contraction shapes on the current state, keep the fastest; returns its index"""
        c = C.c_int()
        self._ck(_lib().dmd_autotune(self._h, int(evals), C.byref(c)))
        return c.value

    @property
    def pair_bytes(self):
        """device bytes of the stored k-pair operators"""
        n = C.c_int64()
        self._ck(_lib().dmd_pair_bytes(self._h, C.byref(n)))
        return n.value

    def sync(self):
        self._ck(_lib().dmd_sync(self._h))

    def timer_start(self):
        self._ck(_lib().dmd_timer(self._h, 0, None))

    def timer_stop(self):
        ms = C.c_double()
        self._ck(_lib().dmd_timer(self._h, 1, C.byref(ms)))
        return ms.value

    def set_profiling(self, on):
        self._ck(_lib().dmd_set_profiling(self._h, 1 if on else 0))

    def profile(self, cls):
        ms, n = C.c_double(), C.c_int64()
        self._ck(_lib().dmd_profile_get(self._h, cls, C.byref(ms), C.byref(n)))
        return ms.value, n.value


class Group:
    """Several LindbladGPU handles of one device stepped together: one CUDA graph launch per RK4 step
    runs every member's step as a parallel branch (separate P sets, e.g. temperatures)."""

    def __init__(self, members):
        self.members = list(members)
        arr = (C.c_void_p * len(self.members))(*[m._h for m in self.members])
        g = C.c_void_p()
        st = _lib().dmd_group_create(arr, len(self.members), C.byref(g))
        if st != 0:
            raise DMDError(st, "dmd_group_create failed")
        self._g = g

    def rk4(self, dt, nsteps):
        st = _lib().dmd_group_rk4(self._g, float(dt), int(nsteps))
        if st != 0:
            msg = "; ".join(_lib().dmd_last_error(m._h).decode() for m in self.members)
            raise DMDError(st, msg)

    def close(self):
        if self._g is not None:
            _lib().dmd_group_destroy(self._g)
            self._g = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PinnedArray:
    """Page-locked host float64 buffer (cudaHostAlloc) exposed as a numpy array."""

    def __init__(self, n):
        p = C.c_void_p()
        st = _lib().dmd_pinned_alloc(int(n) * 8, C.byref(p))
        if st != 0:
            raise DMDError(st, "dmd_pinned_alloc")
        self._p = p
        buf = (C.c_double * int(n)).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=np.float64, count=int(n))

    def free(self):
        if self._p:
            self.array = None
            _lib().dmd_pinned_free(self._p)
            self._p = None
