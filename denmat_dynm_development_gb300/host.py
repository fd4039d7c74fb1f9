"""Python binding of the host library (include/dmd_host.h): DMD's input readers, set-up and run
driver in C++, feeding the GPU ABI."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import HOST_LIB
from . import dmd as _dmd

_L = None

EXPORTS = ["dmdh_load", "dmdh_free", "dmdh_error", "dmdh_info_get", "dmdh_desc", "dmdh_get_dm0", "dmdh_get_f",
           "dmdh_get_smat", "dmdh_get_f_eq", "dmdh_prepare", "dmdh_param", "dmdh_fermi", "dmdh_dm_bpert",
           "dmdh_H_BS", "dmdh_run", "dmdh_ee_desc", "dmdh_rk4_func", "dmdh_tau", "dmdh_report_tau"]


class Info(C.Structure):
    _fields_ = [("nk", C.c_int32), ("nb_dm", C.c_int32), ("bstart", C.c_int32), ("bend", C.c_int32),
                ("nb_total", C.c_int32), ("nv_dm", C.c_int32), ("nkpair", C.c_int64), ("nk_full", C.c_double),
                ("temperature", C.c_double), ("mu", C.c_double), ("prefac_eph", C.c_double), ("cell_size", C.c_double),
                ("cell_size_cmd", C.c_double), ("ob_prefac", C.c_double), ("t0", C.c_double), ("tend", C.c_double),
                ("tstep", C.c_double), ("ode_hstart", C.c_double), ("ode_hmin", C.c_double), ("ode_hmax", C.c_double),
                ("ode_epsabs", C.c_double), ("Bpert", C.c_double * 3), ("B", C.c_double * 3), ("picture", C.c_int32),
                ("expt", C.c_int32), ("has_H", C.c_int32), ("ode_method", C.c_int32), ("eimp_fraction", C.c_double),
                ("mue", C.c_double), ("muh", C.c_double), ("ddmdteq", C.c_int32), ("linear", C.c_int32)]


def _lib():
    global _L
    if _L is None:
        if not os.path.exists(HOST_LIB):
            raise RuntimeError("libdmdhost.so is not built (call __graft_entry__.build())")
        L = C.CDLL(HOST_LIB)
        vp, d = C.c_void_p, C.c_double
        L.dmdh_load.argtypes = [C.c_char_p, C.POINTER(vp)]
        L.dmdh_free.argtypes = [vp]
        L.dmdh_free.restype = None
        L.dmdh_error.restype = C.c_char_p
        L.dmdh_info_get.argtypes = [vp, C.POINTER(Info)]
        L.dmdh_desc.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(_dmd._Desc)]
        L.dmdh_get_dm0.argtypes = [vp, vp]
        L.dmdh_get_f.argtypes = [vp, vp]
        L.dmdh_get_smat.argtypes = [vp, vp]
        L.dmdh_get_f_eq.argtypes = [vp, vp]
        L.dmdh_prepare.argtypes = [vp, vp]
        L.dmdh_ee_desc.argtypes = [vp, C.POINTER(_dmd._EEDesc), C.POINTER(C.c_int32)]
        L.dmdh_param.argtypes = [vp, C.c_char_p, d, C.POINTER(d), C.POINTER(C.c_int)]
        L.dmdh_fermi.argtypes = [d, d, vp, vp, C.c_size_t]
        L.dmdh_dm_bpert.argtypes = [C.c_int32, C.c_int32, vp, vp, vp, d, vp, d, C.c_int32, vp]
        L.dmdh_H_BS.argtypes = [C.c_int32, C.c_int32, vp, vp, vp, C.c_int32, vp]
        L.dmdh_run.argtypes = [C.c_char_p, C.c_int32, C.c_int64]
        L.dmdh_rk4_func.argtypes = [vp, d, d, C.c_int64, vp, C.c_size_t, vp]
        L.dmdh_tau.argtypes = [C.c_int32, C.c_int32, vp, vp, vp, vp, vp, d, d, C.c_int32, C.c_int32, C.c_int32, d, vp]
        L.dmdh_report_tau.argtypes = [vp, C.c_char_p, d, vp, vp]
        _L = L
    return _L


def _ck(st):
    if st != 0:
        raise RuntimeError("dmd host status %d: %s" % (st, _lib().dmdh_error().decode()))


def _arr(ptr, n, dtype):
    if not ptr or n == 0:
        return np.zeros(0, dtype)
    buf = (C.c_char * (n * np.dtype(dtype).itemsize)).from_address(ptr)
    return np.frombuffer(buf, dtype=dtype, count=n)


class System:
    """A DMD input directory loaded and set up by the C++ host library."""

    def __init__(self, directory: str):
        h = C.c_void_p()
        _ck(_lib().dmdh_load(directory.encode(), C.byref(h)))
        self._h = h
        self.info = Info()
        _ck(_lib().dmdh_info_get(h, C.byref(self.info)))
        i = self.info
        self.nk, self.nb_dm = i.nk, i.nb_dm
        nd2 = i.nb_dm * i.nb_dm
        self.dm0 = np.zeros((i.nk, nd2), np.complex128)
        _ck(_lib().dmdh_get_dm0(h, self.dm0.ctypes.data))
        self.f_dm = np.zeros((i.nk, i.nb_dm), np.float64)
        _ck(_lib().dmdh_get_f(h, self.f_dm.ctypes.data))
        self.smat = np.zeros((i.nk, 3, nd2), np.complex128)
        _ck(_lib().dmdh_get_smat(h, self.smat.ctypes.data))
        self.f_eq = None
        if i.ddmdteq or i.linear:
            self.f_eq = np.zeros((i.nk, i.nb_dm), np.float64)
            _ck(_lib().dmdh_get_f_eq(h, self.f_eq.ctypes.data))
        desc = self.desc()
        nb = i.bend - i.bstart
        n4 = int(i.nkpair) * nb ** 4
        self.e_dm = _arr(desc.e_dm, i.nk * i.nb_dm, np.float64).reshape(i.nk, i.nb_dm)
        self.k1st = _arr(desc.k1st, int(i.nkpair), np.uint64)
        self.k2nd = _arr(desc.k2nd, int(i.nkpair), np.uint64)
        self.P1 = _arr(desc.P1, n4, np.complex128)
        self.P2 = _arr(desc.P2, n4, np.complex128)
        self.Hcoh = _arr(desc.Hcoh, i.nk * nd2, np.complex128).reshape(i.nk, nd2) if desc.Hcoh else None
        # the e-e model (eeMode), as dmdh_prepare will attach it
        ed, on = _dmd._EEDesc(), C.c_int32()
        _ck(_lib().dmdh_ee_desc(h, C.byref(ed), C.byref(on)))
        self.ee = None
        if on.value:
            self.ee = dict(kvec=_arr(ed.kvec, i.nk * 3, np.float64).reshape(i.nk, 3), kmesh=tuple(ed.kmesh),
                           U=_arr(ed.U, i.nk * ed.nbw * nb, np.complex128).reshape(i.nk, ed.nbw, nb),
                           f=_arr(ed.f, i.nk * nb, np.float64).reshape(i.nk, nb), GGT=np.array(ed.GGT[:]),
                           cell_size=ed.cell_size, nk_full=ed.nk_full, temperature=ed.temperature,
                           eps_background=ed.eps_background, meff=ed.meff, formula=ed.formula, nfree=ed.nfree,
                           update_screening=ed.update_screening, nv=ed.nv, degauss=ed.degauss, ethr=ed.ethr,
                           antisymmetry=ed.antisymmetry, scale=ed.scale, every_rhs=ed.every_rhs,
                           dynamic=ed.dynamic, ppa_gn=ed.ppa_gn, eppa=ed.eppa, smearing=ed.smearing,
                           two_freqs=ed.two_freqs)

    def desc(self, precision="f64", device=0):
        d = _dmd._Desc()
        p = _dmd.PREC[precision] if isinstance(precision, str) else int(precision)
        _ck(_lib().dmdh_desc(self._h, p, device, C.byref(d)))
        return d

    def y0(self):
        return np.ascontiguousarray(self.dm0).view(np.float64).reshape(-1).copy()

    def param(self, key, unit=1.0):
        v, f = C.c_double(), C.c_int()
        _ck(_lib().dmdh_param(self._h, key.encode(), unit, C.byref(v), C.byref(f)))
        return v.value if f.value else None

    def gpu(self, precision="f64", device=0):
        """A LindbladGPU built from this system (dmd_create on the loaded arrays), with the e-e model
        attached and the equilibrium drift installed when param.in asks for them (dmdh_prepare); with
        alg_linearize the e-e term is already inside the linear operators, with alg_sparseP the handle
        contracts the stored elements only."""
        i = self.info
        g = _dmd.LindbladGPU(nk=i.nk, nb_dm=i.nb_dm, bstart=i.bstart, bend=i.bend, e_dm=self.e_dm,
                             k1st=self.k1st, k2nd=self.k2nd, P1=self.P1, P2=self.P2, prefac_eph=i.prefac_eph,
                             Hcoh=self.Hcoh, picture=i.picture, expt=i.expt, precision=precision, device=device,
                             f_ref=self.f_eq if self.f_eq is not None else self.f_dm, linear=bool(i.linear),
                             ee_flag=self.ee is not None and not i.linear,
                             sparse=bool(self.param("alg_sparseP") or 0))
        try:
            _ck(_lib().dmdh_prepare(self._h, g._h))
        except Exception:
            g.close()
            raise
        return g

    def report_tau(self, directory: str, t: float, y, dydt):
        """DMD's report_tau at (t, y) with dydt the right-hand side there: appends the lines of
        tau_s{x,y,z}_{elec,hole}_tot.out in directory"""
        y = np.ascontiguousarray(y, dtype=np.float64)
        dydt = np.ascontiguousarray(dydt, dtype=np.float64)
        assert y.size == dydt.size == 2 * self.nk * self.nb_dm ** 2
        _ck(_lib().dmdh_report_tau(self._h, directory.encode(), float(t), y.ctypes.data, dydt.ctypes.data))

    def close(self):
        if getattr(self, "_h", None):
            _lib().dmdh_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fermi(T, mu, e):
    e = np.ascontiguousarray(e, dtype=np.float64)
    f = np.empty_like(e)
    _ck(_lib().dmdh_fermi(T, mu, e.ctypes.data, f.ctypes.data, e.size))
    return f


def dm_bpert(smat, e, f, T, Bpert, t0=0.0, picture=0):
    smat = np.ascontiguousarray(smat, dtype=np.complex128)
    e = np.ascontiguousarray(e, dtype=np.float64)
    f = np.ascontiguousarray(f, dtype=np.float64)
    nk, nb = e.shape
    B = np.ascontiguousarray(Bpert, dtype=np.float64)
    dm = np.zeros((nk, nb * nb), np.complex128)
    _ck(_lib().dmdh_dm_bpert(nk, nb, smat.ctypes.data, e.ctypes.data, f.ctypes.data, T, B.ctypes.data, t0, picture,
                             dm.ctypes.data))
    return dm


def H_BS(smat, B, e, picture=0):
    smat = np.ascontiguousarray(smat, dtype=np.complex128)
    e = np.ascontiguousarray(e, dtype=np.float64)
    nk, nb = e.shape
    Bv = np.ascontiguousarray(B, dtype=np.float64)
    H = np.zeros((nk, nb * nb), np.complex128)
    _ck(_lib().dmdh_H_BS(nk, nb, smat.ctypes.data, Bv.ctypes.data, e.ctypes.data, picture, H.ctypes.data))
    return H


def tau(obs, e, f, dm, ddmdt, t, dt, picture=0, bstart=0, bend=None, prefac=1.0):
    """Instantaneous lifetimes (tau by finite difference over dt, without precession, with it; atomic
    units) of one observable (complex [nk][nb^2]) over bands [bstart, bend) from the state dm and
    its time derivative ddmdt (complex [nk][nb^2])"""
    e = np.ascontiguousarray(e, dtype=np.float64)
    nk, nb = e.shape
    obs, dm, ddmdt = (np.ascontiguousarray(a, dtype=np.complex128) for a in (obs, dm, ddmdt))
    f = np.ascontiguousarray(f, dtype=np.float64)
    assert obs.size == dm.size == ddmdt.size == nk * nb * nb and f.size == nk * nb
    out = np.zeros(3)
    _ck(_lib().dmdh_tau(nk, nb, obs.ctypes.data, e.ctypes.data, f.ctypes.data, dm.ctypes.data, ddmdt.ctypes.data,
                        float(t), float(dt), int(picture), int(bstart), int(nb if bend is None else bend),
                        float(prefac), out.ctypes.data))
    return out


def rk4_func(handle, t, dt, nsteps, y, work):
    """Fixed-step RK4 driven from the host over the GSL-callback entry dmd_func (4 calls per step,
    host copies in and out of each call): y (float64, 2 nk nb_dm^2) is advanced in place; work holds
    5 y.size doubles (page-locked arrays make the copies direct)."""
    assert y.dtype == np.float64 and y.flags.c_contiguous and work.dtype == np.float64 and work.size >= 5 * y.size
    _ck(_lib().dmdh_rk4_func(handle._h, float(t), float(dt), int(nsteps), y.ctypes.data, y.size, work.ctypes.data))


def run(directory: str, precision="f64", nsteps_max=-1):
    """DMD's time loop (evolve_gsl / evolve_euler / RK4) on the GPU, writing the S files into directory."""
    p = _dmd.PREC[precision] if isinstance(precision, str) else int(precision)
    _ck(_lib().dmdh_run(directory.encode(), p, int(nsteps_max)))
