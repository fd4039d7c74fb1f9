"""ORACLE (test infrastructure only): Python side of the CPU restatement in dmd_oracle.c.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module, always as
the side the GPU results are compared with (or timed beside). It reads a DMD input directory (param.in + ldbd_data/) the way the reference's
constructors do and calls the C restatement through ctypes.

Setup statements restated here (reference file:line):
  * param.in parsing -- parameters::map_input (parameters.cpp:591-623) and get() (:530-548),
    including the key = trim(substr(0, '=' position - 1)) convention;
  * ldbd_size.dat / ldbd_R.dat / ldbd_ek.bin / ldbd_smat.bin / kpair / P readers --
    electron.cpp:100-314, lattice.h:48-56, ElectronPhonon.cpp:132-253, parameters.cpp:7-23;
  * Fermi occupations -- electron::fermi (electron.h:119-124) with mu = (mu_file/eV)*eV as get()
    returns it;
  * e-imp fold P += |n_i V_cell| * P_D1 -- ElectronImpurity.cpp:3-49 and ElectronPhonon.cpp:44-113;
  * initial state -- electron::compute_dm_Bpert_1st (electron.cpp:62-98) then
    singdenmat_k::init_dm (DenMat.cpp:65-81);
  * coherent Hamiltonian -- electron::set_H_BS (electron.cpp:19-42), singdenmat_k::init_Hcoh
    (DenMat.cpp:7-28);
  * observable prefactor 1/(nk_full * cell_size_cmd) -- observable.h:54, lattice.h:27-36.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from dataclasses import dataclass
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRCS = [os.path.join(HERE, "dmd_oracle.c"), os.path.join(HERE, "gsl_rkf45.c"),
        os.path.join(HERE, "ref_shim", "cblas_shim.c")]

# comm/Units.h
eV = 1.0 / 27.21138505
Joule = 1.0 / 4.35974434e-18
Angstrom = 1.0 / 0.5291772
meter = 1e10 * Angstrom
kg = 1.0 / 9.10938291e-31
Newton = Joule / meter
sec = math.sqrt((kg * meter) / Newton)
fs = sec * 1.0e-15
Tesla2au = 1.0 / 2.3505175675871e5
bohr2cm = 5.291772109038e-9


def build(force: bool = False) -> str:
    """Compile liboracle.so (gcc, -ffp-contract=off so rounding is host independent)."""
    newest = max(os.path.getmtime(s) for s in SRCS)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = ["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I", os.path.join(HERE, "ref_shim", "include"),
               "-o", LIB + ".tmp"] + SRCS + ["-lm"]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _lib.orc_rhs.argtypes = [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p]
        _lib.orc_ee_P.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                  C.c_void_p, C.c_void_p]
        _lib.orc_ee_P.restype = None
        _lib.orc_ee_rebuild.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]
        _lib.orc_ee_rebuild.restype = None
        _lib.orc_ee_rpa_table.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        _lib.orc_ee_rpa_table.restype = None
        _lib.orc_rhs_parts.argtypes = [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_rk4.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_long, C.c_void_p, C.c_long, C.c_void_p, C.c_void_p]
        _lib.orc_rkf45.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                   C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_long]
        _lib.orc_rkf45.restype = C.c_int
        _lib.orc_euler.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_long, C.c_void_p]
        _lib.orc_measure.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p,
                                     C.c_double, C.c_int, C.c_void_p, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _lib.orc_sys_size.restype = C.c_size_t
        _lib.orc_window_in.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_pairs_partial.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_int64,
                                           C.c_int64, C.c_void_p, C.c_void_p]
        _lib.orc_rhs_from_partials.argtypes = [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_fermi.argtypes = [C.c_double, C.c_double, C.c_void_p, C.c_void_p, C.c_size_t]
        _lib.orc_compute_nfree.argtypes = [C.c_int, C.c_double, C.c_double, C.c_void_p, C.c_int, C.c_int, C.c_int]
        _lib.orc_compute_nfree.restype = C.c_double
        _lib.orc_find_mu_bisect.argtypes = [C.c_double, C.c_int, C.c_double, C.c_double, C.c_double, C.c_void_p,
                                            C.c_int, C.c_int, C.c_int]
        _lib.orc_find_mu_bisect.restype = C.c_double
        _lib.orc_set_dm_eq.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_double, C.c_void_p, C.c_int,
                                       C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        _lib.orc_set_dm_eq.restype = C.c_int
        _lib.orc_compute_ddmdt_eq.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_compute_ddmdt_eq.restype = None
        _lib.orc_lsc_add.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_lsc_add.restype = None
        _lib.orc_lsc_add2.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        _lib.orc_lsc_add2.restype = None
        _lib.orc_ee_P3P6.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p]
        _lib.orc_ee_P3P6.restype = None
        for n in ("orc_lsc_add_p3p4", "orc_lsc_add_p5p6"):
            getattr(_lib, n).argtypes = [C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p]
            getattr(_lib, n).restype = None
        _lib.orc_lsc_diag.argtypes = [C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_lsc_diag.restype = None
    return _lib


class _Sys(C.Structure):
    _fields_ = [("nk", C.c_int), ("nb_dm", C.c_int), ("bstart", C.c_int), ("bend", C.c_int), ("npair", C.c_int64),
                ("k1st", C.c_void_p), ("k2nd", C.c_void_p), ("P1", C.c_void_p), ("P2", C.c_void_p),
                ("e_dm", C.c_void_p), ("prefac_eph", C.c_double), ("Hcoh", C.c_void_p),
                ("picture_schrodinger", C.c_int), ("expt", C.c_int), ("ddmdt_eq", C.c_void_p), ("scatt_enable", C.c_int),
                ("linear", C.c_int), ("f_lin", C.c_void_p), ("ee", C.c_void_p), ("sparse", C.c_int),
                ("thr_sparse", C.c_double)]


class _EE(C.Structure):
    """orc_ee (dmd_oracle.c): the e-e model of eeMode = Pee_update with static screening"""
    _fields_ = [("nb", C.c_int), ("nbw", C.c_int), ("kvec", C.c_void_p), ("kmesh", C.c_int * 3), ("U", C.c_void_p),
                ("GGT", C.c_double * 9), ("cell_size", C.c_double), ("nk_full", C.c_double), ("T", C.c_double),
                ("eps", C.c_double), ("meff", C.c_double), ("formula", C.c_int), ("nfree", C.c_double),
                ("update_screening", C.c_int), ("nv", C.c_int), ("degauss", C.c_double), ("ethr", C.c_double),
                ("antisym", C.c_int), ("scale", C.c_double), ("inside", C.c_int), ("P1base", C.c_void_p),
                ("P2base", C.c_void_p), ("P1eff", C.c_void_p), ("P2eff", C.c_void_p), ("P1ee", C.c_void_p),
                ("P2ee", C.c_void_p), ("f_setup", C.c_void_p), ("vq_rpa", C.c_void_p), ("dynamic", C.c_int),
                ("ppa_gn", C.c_int), ("eppa", C.c_double), ("smearing", C.c_double), ("two_freqs", C.c_int),
                ("Aq_ppa", C.c_void_p), ("Eq2_ppa", C.c_void_p)]


EE_FORMULAS = {"unscreened": 0, "debye": 1, "Bechstedt": 2, "RPA": 3, "lindhard": 4}


def ggt_of(R):
    """lattice::GGT = Gvec Gvec^T with Gvec = 2 pi inv(R) (lattice.h:41-42), in the operation order of
    comm/matrix3.h (inv = adjugate / det with det = box of the rows, products summed from k = 0) and
    comm/vector3.h (cross, dot)."""
    r = [[float(R[i][j]) for j in range(3)] for i in range(3)]

    def cross(a, b):
        return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]

    def dot(a, b):
        return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]

    det = dot(r[0], cross(r[1], r[2]))
    cols = [cross(r[1], r[2]), cross(r[2], r[0]), cross(r[0], r[1])]
    s = 1. / det
    inv = [[cols[j][i] * s for j in range(3)] for i in range(3)]
    G = [[inv[i][j] * (2. * math.pi) for j in range(3)] for i in range(3)]
    out = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            acc = 0.0
            for k in range(3):
                acc += G[i][k] * G[j][k]
            out[i, j] = acc
    return out


class EEModel:
    """The e-e model's inputs (what elecelec_model / coulomb_model hold) and its operator buffers.
    P1eff, P2eff are the system's P1, P2: P_base + scale P_ee, rebuilt in place from rho."""

    def __init__(self, *, nb, kvec, kmesh, U, GGT, cell_size, nk_full, T, eps, meff, formula, nfree, update_screening,
                 nv, degauss, ethr, antisym, scale, inside, P1base, P2base, f_setup=None, e_window=None,
                 dynamic="static", ppamodel="gn", eppa=0.0, smearing=0.0, two_freqs=0):
        self.kvec = np.ascontiguousarray(kvec, np.float64)
        self.U = np.ascontiguousarray(U, np.complex128)
        self.P1base = np.ascontiguousarray(P1base, np.complex128)
        self.P2base = np.ascontiguousarray(P2base, np.complex128)
        self.P1eff = self.P1base.copy()
        self.P2eff = self.P2base.copy()
        self.P1ee = np.zeros_like(self.P1base)
        self.P2ee = np.zeros_like(self.P2base)
        self.nb, self.nbw = int(nb), int(self.U.shape[1])
        self.kmesh = tuple(int(x) for x in kmesh)
        self.GGT = np.ascontiguousarray(GGT, np.float64).reshape(9)
        self.cell_size, self.nk_full, self.T, self.eps, self.meff = cell_size, nk_full, T, eps, meff
        self.formula = EE_FORMULAS[formula] if isinstance(formula, str) else int(formula)
        self.update_screening, self.nv = int(update_screening), int(nv)
        self.degauss, self.ethr, self.antisym, self.scale = degauss, ethr, int(antisym), scale
        self.inside = int(inside)
        self.f_setup = None if f_setup is None else np.ascontiguousarray(f_setup, np.float64)
        self.vq_rpa = np.zeros(int(np.prod(self.kmesh)), np.float64) if self.formula >= 3 else None
        # dynamic screening (Scatt_Param.h:20-49, Coulomb_Model.h:520-530, 572-575): the plasmon-pole
        # approximation with RPA / Lindhard screening only; eppa defaults to the plasma frequency of
        # the set-up density, the smearing to 0.5 T except for Godby-Needs
        if dynamic not in ("static", "ppa"):
            raise ValueError("the oracle restates static and ppa screening only")
        self.dynamic = 1 if dynamic == "ppa" else 0
        if self.dynamic and self.formula < 3:
            raise ValueError("dynamic screening needs RPA or lindhard (the reference refuses the other formulas)")
        self.ppa_gn = 1 if ppamodel == "gn" else 0
        if self.dynamic and eppa == 0:
            eppa = math.sqrt(4 * math.pi * nfree / meff / eps)
        if not (self.dynamic and self.ppa_gn):
            smearing = 0.5 * T if smearing <= 0 else smearing
        self.eppa, self.smearing, self.two_freqs = float(eppa), float(smearing), int(two_freqs)
        nm = int(np.prod(self.kmesh)) if self.dynamic else 1
        self.Aq_ppa = np.zeros(nm, np.complex128)
        self.Eq2_ppa = np.zeros(nm, np.complex128)
        self.c = _EE(nb=self.nb, nbw=self.nbw, kvec=self.kvec.ctypes.data, kmesh=(C.c_int * 3)(*self.kmesh),
                     U=self.U.ctypes.data, GGT=(C.c_double * 9)(*self.GGT), cell_size=cell_size, nk_full=nk_full, T=T,
                     eps=eps, meff=meff, formula=self.formula, nfree=nfree, update_screening=self.update_screening,
                     nv=self.nv, degauss=degauss, ethr=ethr, antisym=self.antisym, scale=scale, inside=self.inside,
                     P1base=self.P1base.ctypes.data, P2base=self.P2base.ctypes.data, P1eff=self.P1eff.ctypes.data,
                     P2eff=self.P2eff.ctypes.data, P1ee=self.P1ee.ctypes.data, P2ee=self.P2ee.ctypes.data,
                     f_setup=None if self.f_setup is None else self.f_setup.ctypes.data,
                     vq_rpa=None if self.vq_rpa is None else self.vq_rpa.ctypes.data, dynamic=self.dynamic,
                     ppa_gn=self.ppa_gn, eppa=self.eppa, smearing=self.smearing, two_freqs=self.two_freqs,
                     Aq_ppa=self.Aq_ppa.ctypes.data, Eq2_ppa=self.Eq2_ppa.ctypes.data)
        if self.formula >= 3:  # the static RPA / Lindhard screening of the set-up (Coulomb_Model.h:690-826)
            if self.f_setup is None or e_window is None:
                raise ValueError("RPA / lindhard screening needs the set-up occupations and energies")
            ew = np.ascontiguousarray(e_window, np.float64)
            lib().orc_ee_rpa_table(C.addressof(self.c), C.c_int(self.kvec.shape[0]), ew.ctypes.data)

    @property
    def nfree(self):
        return self.c.nfree

    @nfree.setter
    def nfree(self, v):
        self.c.nfree = v


class _Meas(C.Structure):
    _fields_ = [("obs", C.c_void_p), ("obs_kstride", C.c_size_t), ("f", C.c_void_p), ("prefac", C.c_double),
                ("bs", C.c_int), ("be", C.c_int)]


def _ptr(a):
    return None if a is None else a.ctypes.data


# ------------------------------------------------------------------------------------------------
# param.in
# ------------------------------------------------------------------------------------------------
def parse_param_in(path: str) -> dict:
    """parameters::map_input (parameters.cpp:591-623)."""
    def trim(s):
        s = s.lstrip(" ")
        return s.rstrip(" \n\r\t")
    out, last_key, b_join = {}, "", False
    with open(path) as f:
        for line in f.read().split("\n"):
            b_will_join = False
            b_joined = False
            line2 = trim(line)
            if line[:1] == "#":
                continue
            if line2 and line2[-1] == "\\":
                b_will_join = True
                line2 = line2[:-1] + " "
            if b_join:
                out[last_key] += " " + line2
                b_joined = True
            b_join = b_will_join
            if not b_joined:
                eq = line2.find("=")
                if eq < 0:
                    continue
                last_key = trim(line2[:max(eq - 1, 0)])
                out[last_key] = trim(line2[eq + 1:])
    return out


def _atof(s: str) -> float:
    """C atof: longest numeric prefix, 0 when none."""
    s = s.strip()
    best = 0.0
    for i in range(len(s), 0, -1):
        try:
            best = float(s[:i])
            return best
        except ValueError:
            continue
    return best


def pget(m: dict, key: str, default: float, unit: float = 1.0) -> float:
    """parameters::get (parameters.cpp:530-548)."""
    if key in m:
        return _atof(m[key]) * unit
    return default * unit


# ------------------------------------------------------------------------------------------------
# ldbd_data
# ------------------------------------------------------------------------------------------------
def read_size(d: str) -> dict:
    with open(os.path.join(d, "ldbd_data", "ldbd_size.dat")) as f:
        lines = f.read().split("\n")
    l2 = [int(x) for x in lines[1].split("#")[0].split()]
    l3 = lines[2].split("#")[0].split()
    info = dict(nb=l2[0], nv=l2[1], bStart_dm=l2[2], bEnd_dm=l2[3], bStart_eph=l2[4], bEnd_eph=l2[5],
                nk_full=float(l3[0]), nk=int(l3[1]), kmesh=tuple(int(x) for x in l3[2:5]),
                nkpair=int(lines[3].split("#")[0].split()[0]),
                temperature=float(lines[5].split("#")[0].split()[0]),
                mu=float(lines[6].split("#")[0].split()[2]),
                nb_wannier=l2[6] if len(l2) > 6 else l2[0])
    dg = lines[7].split("#")[0].split() if len(lines) > 7 else []
    info["degauss"] = float(dg[0]) if dg else 0.0
    info["ndegauss"] = float(dg[1]) if len(dg) > 1 else 0.0
    return info


def read_R(d: str) -> np.ndarray:
    with open(os.path.join(d, "ldbd_data", "ldbd_R.dat")) as f:
        tok = f.read().split()
    dim = int(tok[0])
    R = np.array([float(x) for x in tok[1:10]]).reshape(3, 3)
    return dim, R


def det3(R):
    """matrix3 determinant by cofactor expansion along the first row."""
    return (R[0, 0] * (R[1, 1] * R[2, 2] - R[1, 2] * R[2, 1]) - R[0, 1] * (R[1, 0] * R[2, 2] - R[1, 2] * R[2, 0])
            + R[0, 2] * (R[1, 0] * R[2, 1] - R[1, 1] * R[2, 0]))


def fermi(T, mu, e):
    """electron::fermi (electron.h:119-124), elementwise, evaluated in C with libm's exp."""
    e = np.ascontiguousarray(e, dtype=np.float64)
    out = np.empty_like(e)
    lib().orc_fermi(C.c_double(T), C.c_double(mu), C.c_void_p(e.ctypes.data), C.c_void_p(out.ctypes.data),
                    C.c_size_t(e.size))
    return out


def dm_bpert(smat, e, f, T, Bpert, t0=0.0, picture=0):
    """Initial state: electron::compute_dm_Bpert_1st (electron.cpp:62-98) followed by
    singdenmat_k::init_dm (DenMat.cpp:65-81), as load() builds it. smat [nk][3][nb^2] complex,
    e, f [nk][nb]; returns complex [nk][nb^2]."""
    _setup_prototypes()
    smat = np.ascontiguousarray(smat, dtype=np.complex128)
    e = np.ascontiguousarray(e, dtype=np.float64)
    f = np.ascontiguousarray(f, dtype=np.float64)
    B = np.ascontiguousarray(Bpert, dtype=np.float64)
    nk, nb = e.shape
    L = lib()
    dmB = np.zeros((nk, nb * nb), np.complex128)
    L.orc_dm_bpert(C.c_int(nk), C.c_int(nb), C.c_void_p(smat.ctypes.data), C.c_void_p(e.ctypes.data),
                   C.c_void_p(f.ctypes.data), C.c_double(T), C.c_void_p(B.ctypes.data), C.c_double(t0),
                   C.c_int(picture), C.c_void_p(dmB.ctypes.data))
    dm0 = np.zeros_like(dmB)
    L.orc_init_dm(C.c_int(nk), C.c_int(nb), C.c_void_p(dmB.ctypes.data), C.c_void_p(dm0.ctypes.data))
    return dm0


@dataclass
class OracleSystem:
    nk: int
    nb_dm: int
    bstart: int
    bend: int
    npair: int
    e_dm: np.ndarray
    f_dm: np.ndarray
    k1st: np.ndarray
    k2nd: np.ndarray
    P1: np.ndarray
    P2: np.ndarray
    prefac_eph: float
    Hcoh: Optional[np.ndarray]
    smat: np.ndarray
    dm0: np.ndarray
    picture_schrodinger: int
    expt: int
    t0: float
    tstep: float
    tend: float
    temperature: float
    mu: float
    nk_full: float
    ob_prefac: float
    ode: dict
    params: dict
    nv_dm: int = 0
    mue: float = 0.0
    muh: float = 0.0
    f_eq: Optional[np.ndarray] = None        # [nk][nb_dm] with alg_ddmdteq or alg_linearize
    ddmdt_eq: Optional[np.ndarray] = None    # [nk][nb^2] window, subtracted from the scattering term
    linear: bool = False                     # alg_linearize: P1, P2 hold Lscij, Lscji
    f_lin: Optional[np.ndarray] = None       # [nk][nb] window f_eq of the linearization
    ee: Optional[EEModel] = None             # eeMode = Pee_update: P1, P2 are ee.P1eff, ee.P2eff
    sparse: bool = False                     # alg.sparseP: P contracted as sparse_mat (sparse_zgemm)
    lin_ee: Optional[tuple] = None           # linearized e-e source: P1ee, P2ee, P3..P6 (times scale_ee)
    thr_sparse: float = 1e-40                # alg.thr_sparseP

    def cstruct(self):
        s = _Sys(nk=self.nk, nb_dm=self.nb_dm, bstart=self.bstart, bend=self.bend, npair=self.npair,
                 k1st=_ptr(self.k1st), k2nd=_ptr(self.k2nd), P1=_ptr(self.P1), P2=_ptr(self.P2), e_dm=_ptr(self.e_dm),
                 prefac_eph=self.prefac_eph, Hcoh=_ptr(self.Hcoh), picture_schrodinger=self.picture_schrodinger,
                 expt=self.expt, ddmdt_eq=_ptr(self.ddmdt_eq), scatt_enable=1, linear=1 if self.linear else 0,
                 f_lin=_ptr(self.f_lin), ee=C.addressof(self.ee.c) if self.ee is not None else None,
                 sparse=1 if self.sparse else 0, thr_sparse=self.thr_sparse)
        return s

    @property
    def ny(self):
        return 2 * self.nk * self.nb_dm * self.nb_dm


def _ee_model_of(pm, sz, dd, R, nk, nb, nb_dm, bstart, bend, e_dm, f_dm, nv_dm, T, cell_size, nfree, P1, P2):
    """The e-e model's inputs as elecelec_model / coulomb_model read them (ElecElec_Model.h:22-37,
    Coulomb_Model.h:394-450): U, k-points, reciprocal metric, screening parameters."""
    nbw = sz["nb_wannier"]
    nb_eph = sz["bEnd_eph"] - sz["bStart_eph"]
    U = np.fromfile(os.path.join(dd, "ldbd_Umat.bin"), dtype=np.complex128).reshape(nk, nbw, nb_eph)
    kvec = np.fromfile(os.path.join(dd, "ldbd_kvec.bin"), dtype=np.float64).reshape(nk, 3)
    degauss, ndegauss = sz["degauss"], sz["ndegauss"]
    degauss = pget(pm, "degauss", degauss / eV, eV)
    ndegauss = pget(pm, "ndegauss", ndegauss)
    scale_scatt = pget(pm, "scale_scatt", 1.0)
    return EEModel(nb=nb, kvec=kvec, kmesh=sz["kmesh"], U=U, GGT=ggt_of(R), cell_size=cell_size,
                   nk_full=sz["nk_full"], T=T, eps=pget(pm, "epsilon_background", 1.0),
                   meff=pget(pm, "meff_screening", 1.0), formula=pm.get("scrFormula", "RPA"), nfree=nfree,
                   update_screening=int(pget(pm, "update_screening", 1)), nv=nv_dm - bstart,
                   degauss=pget(pm, "degauss_ee", degauss / eV, eV), ethr=degauss * ndegauss,
                   antisym=int(pget(pm, "ee_antisymmetry", 0)), scale=pget(pm, "scale_ee", scale_scatt),
                   inside=pget(pm, "freq_update_ee_model", 0) < 0, P1base=P1, P2base=P2,
                   f_setup=f_dm[:, bstart:bend], e_window=e_dm[:, bstart:bend],
                   dynamic=pm.get("dynamic_screening", "static"), ppamodel=pm.get("ppamodel", "gn"),
                   eppa=pget(pm, "eppa_screening", 0.0), smearing=pget(pm, "smearing_screening", 0.0, eV),
                   two_freqs=int(pget(pm, "dynamic_screening_ee_two_freqs", 0)))


def _ee_linear_terms(pm, sz, dd, R, nk, nb, nb_dm, bstart, bend, npair, k1, k2, e_dm, f_dm, f_lin, nv_dm, T,
                     cell_size, nfree, smat, dm0, schrod, expt, t0, mu):
    """The e-e source of the linear operators (electronphonon::set_Lsc, ElectronPhonon_linear.cpp:
    17-22, 44-100): the screening density from f_eq when the model updates it (coulomb_model::init,
    Coulomb_Model.h:532-544), P_ee at f_eq (calc_P with ee_model->f = f_eq) and, unless eeMode =
    Pee_fixed_at_eq, P3..P6 (ElecElec_Model_linear.cpp), each times scale_ee."""
    nb4 = nb ** 4
    if pm.get("dynamic_screening", "static") != "static":
        raise ValueError("the linearized e-e source is restated with static screening only")
    zero = np.zeros(npair * nb4, np.complex128)
    ee = _ee_model_of(pm, sz, dd, R, nk, nb, nb_dm, bstart, bend, e_dm, f_dm, nv_dm, T, cell_size, nfree, zero, zero)
    n = nfree
    if ee.update_screening:
        fw = f_lin
        n = float(sum((1 - fw[ik, b]) if b < ee.nv else fw[ik, b] for ik in range(nk) for b in range(nb)))
        n /= (sz["nk_full"] * cell_size)
    tmp = OracleSystem(nk=nk, nb_dm=nb_dm, bstart=bstart, bend=bend, npair=npair, e_dm=e_dm, f_dm=f_dm, k1st=k1,
                       k2nd=k2, P1=zero, P2=zero, prefac_eph=2 * math.pi / sz["nk_full"], Hcoh=None, smat=smat,
                       dm0=dm0, picture_schrodinger=schrod, expt=expt, t0=t0, tstep=0.0, tend=0.0, temperature=T,
                       mu=mu, nk_full=sz["nk_full"], ob_prefac=1.0, ode={}, params={})
    cs = tmp.cstruct()
    L = lib()
    fl = np.ascontiguousarray(f_lin)
    L.orc_ee_P(C.addressof(ee.c), C.addressof(cs), None, None, fl.ctypes.data, C.c_double(n), ee.P1ee.ctypes.data,
               ee.P2ee.ctypes.data)
    P = [np.zeros(npair * nb4, np.complex128) for _ in range(4)]
    fixed = pm.get("eeMode", "none") == "Pee_fixed_at_eq"
    if not fixed:
        L.orc_ee_P3P6(C.addressof(ee.c), C.addressof(cs), fl.ctypes.data, C.c_double(n), *[x.ctypes.data for x in P])
    out = [ee.P1ee.copy(), ee.P2ee.copy()] + P
    if ee.scale != 1.0:
        out = [x * complex(ee.scale, 0) for x in out]
    return tuple(out) + (bool(ee.antisym), fixed)


def load(d: str) -> OracleSystem:
    """Read param.in + ldbd_data/ in directory d and build the state DMD has after set-up."""
    pm = parse_param_in(os.path.join(d, "param.in"))
    sz = read_size(d)
    nk, nbt = sz["nk"], sz["nb"]
    nb_dm = sz["bEnd_dm"] - sz["bStart_dm"]
    bstart, bend = sz["bStart_eph"] - sz["bStart_dm"], sz["bEnd_eph"] - sz["bStart_dm"]
    nb = bend - bstart
    T = sz["temperature"]
    mu = pget(pm, "mu", sz["mu"] / eV, eV)
    dd = os.path.join(d, "ldbd_data")
    e = np.fromfile(os.path.join(dd, "ldbd_ek.bin"), dtype=np.float64).reshape(nk, nbt)
    scissor = pget(pm, "scissor", 0.0, eV)
    if scissor != 0:
        e[:, sz["nv"]:] += scissor
    e_dm = np.ascontiguousarray(e[:, sz["bStart_dm"]:sz["bEnd_dm"]])
    nv_dm = max(sz["nv"] - sz["bStart_dm"], 0)  # electron.cpp:114
    dim, R = read_R(d)
    dim = int(pget(pm, "dim", dim))
    vol = abs(det3(R))
    cell_size = vol if dim == 3 else (vol / R[2, 2] if dim == 2 else (R[2, 2] if dim == 1 else 1.0))
    nimp = 0
    while pget(pm, "impurity_density" + ("" if nimp == 0 else str(nimp + 1)), 0.0) != 0:
        nimp += 1
    mu, gs, nfree = set_mu_and_n(pm, e, e_dm, sz, nv_dm, T, mu, cell_size, dim)
    f = fermi(T, mu, e)
    f_dm = np.ascontiguousarray(f[:, sz["bStart_dm"]:sz["bEnd_dm"]])
    smat = np.fromfile(os.path.join(dd, "ldbd_smat.bin"), dtype=np.complex128).reshape(nk, 3, nb_dm * nb_dm)
    npair = sz["nkpair"]
    k1 = np.fromfile(os.path.join(dd, "ldbd_kpair_k1st.bin"), dtype=np.uint64)
    k2 = np.fromfile(os.path.join(dd, "ldbd_kpair_k2nd.bin"), dtype=np.uint64)
    assert k1.size == npair and k2.size == npair, "ldbd_kpair size does not match nkpair"
    nb4 = nb ** 4
    P1 = np.fromfile(os.path.join(dd, "ldbd_P1_lindblad.bin"), dtype=np.complex128)
    P2 = np.fromfile(os.path.join(dd, "ldbd_P2_lindblad.bin"), dtype=np.complex128)
    assert P1.size == npair * nb4 and P2.size == npair * nb4, "ldbd_P size does not match"
    scale_scatt = pget(pm, "scale_scatt", 1.0)
    scale_eph = pget(pm, "scale_eph", scale_scatt)
    if scale_eph != 1.0:
        P1 = P1 * complex(scale_eph, 0)
        P2 = P2 * complex(scale_eph, 0)
    linear = int(pget(pm, "alg_linearize", 0)) != 0
    imps = []  # impurity operators times |n_i V| (electronimpurity::read_ldbd_imp_P, ElectronImpurity.cpp:38-39)
    ni = pget(pm, "impurity_density", 0.0, bohr2cm ** dim)
    if ni != 0:
        fraction = abs(ni * cell_size)
        Q1 = np.fromfile(os.path.join(dd, "ldbd_P1_lindblad_D1.bin"), dtype=np.complex128)
        Q2 = np.fromfile(os.path.join(dd, "ldbd_P2_lindblad_D1.bin"), dtype=np.complex128)
        if linear:
            imps.append((Q1 * fraction, Q2 * fraction))
        else:
            P1 = P1 + Q1 * fraction
            P2 = P2 + Q2 * fraction
    picture = pm.get("alg_picture", "interaction")
    schrod = 1 if picture in ("schrodinger", "non-interaction") else 0
    expt = int(pget(pm, "alg_expt", 1.0))
    t0 = pget(pm, "t0", 0.0, fs)
    Bpert = np.array([pget(pm, "Bxpert", 0.0, Tesla2au), pget(pm, "Bypert", 0.0, Tesla2au), pget(pm, "Bzpert", 0.0, Tesla2au)])
    B = np.array([pget(pm, "Bx", 0.0, Tesla2au), pget(pm, "By", 0.0, Tesla2au), pget(pm, "Bz", 0.0, Tesla2au)])
    L = lib()
    dmB = np.zeros((nk, nb_dm * nb_dm), np.complex128)
    L.orc_dm_bpert(C.c_int(nk), C.c_int(nb_dm), C.c_void_p(smat.ctypes.data), C.c_void_p(e_dm.ctypes.data),
                   C.c_void_p(f_dm.ctypes.data), C.c_double(T), C.c_void_p(Bpert.ctypes.data), C.c_double(t0),
                   C.c_int(schrod), C.c_void_p(dmB.ctypes.data))
    dm0 = np.zeros_like(dmB)
    L.orc_init_dm(C.c_int(nk), C.c_int(nb_dm), C.c_void_p(dmB.ctypes.data), C.c_void_p(dm0.ctypes.data))
    Hcoh = None
    if math.sqrt(float((B * B).sum())) > 1e-10:
        Hcoh = np.zeros((nk, nb_dm * nb_dm), np.complex128)
        L.orc_H_BS(C.c_int(nk), C.c_int(nb_dm), C.c_void_p(smat.ctypes.data), C.c_void_p(B.ctypes.data),
                   C.c_void_p(e_dm.ctypes.data), C.c_int(schrod), C.c_void_p(Hcoh.ctypes.data))
    tstep = pget(pm, "tstep", 1.0, fs)
    ode = dict(hstart=pget(pm, "ode_hstart", 1e-3, fs), hmin=pget(pm, "ode_hmin", 0.0, fs),
               hmax=pget(pm, "ode_hmax", tstep / fs, fs), epsabs=pget(pm, "ode_epsabs", 1e-8))
    cell_size_cmd = cell_size * bohr2cm ** dim
    f_eq = ddmdt_eq = None
    mue = muh = mu
    f_lin = None
    if int(pget(pm, "alg_ddmdteq", 0)) or linear:
        # DensityMatrix_Dynamics.h:58-63: set_dm_eq on the initial state, then compute_ddmdt_eq or set_Lsc
        f_eq = np.zeros((nk, nb_dm))
        mus = np.array([mu, mu])
        g = np.array(gs)
        rc = L.orc_set_dm_eq(nk, nb_dm, nv_dm, dm0.ctypes.data, T, e_dm.ctypes.data, nimp, g.ctypes.data,
                             int(pget(pm, "DEBUG", 0)), mus.ctypes.data, f_eq.ctypes.data)
        assert rc == 0, "carrier_bvk_ex is undefined for this input (impurities with zero ground-state carriers)"
        mue, muh = float(mus[0]), float(mus[1])
    if linear:
        # electronphonon::set_Lsc (ElectronPhonon_linear.cpp:3-31): e-ph operators, then each impurity's,
        # then Lscii onto the diagonal pairs
        f_lin = np.ascontiguousarray(f_eq[:, bstart:bend])
        nb4 = nb ** 4
        Lii = np.zeros(nk * nb4, np.complex128)
        Lij = np.zeros(npair * nb4, np.complex128)
        Lji = np.zeros(npair * nb4, np.complex128)
        srcs = [(np.ascontiguousarray(P1), np.ascontiguousarray(P2))] + [
            (np.ascontiguousarray(a), np.ascontiguousarray(b)) for a, b in imps]
        for a, b in srcs:
            L.orc_lsc_add(nk, nb, npair, k1.ctypes.data, k2.ctypes.data, a.ctypes.data, b.ctypes.data, f_lin.ctypes.data,
                          Lii.ctypes.data, Lij.ctypes.data, Lji.ctypes.data)
        lin_ee = None
        if pm.get("eeMode", "none") != "none":  # add_Lsc_contrib("ee"), ElectronPhonon_linear.cpp:17-22, 44-100
            lin_ee = _ee_linear_terms(pm, sz, dd, R, nk, nb, nb_dm, bstart, bend, npair, k1, k2, e_dm, f_dm, f_lin,
                                      nv_dm, T, cell_size, nfree, smat, dm0, schrod, expt, t0, mu)
            P1ee, P2ee, P3, P4, P5, P6, antisym, fixed = lin_ee
            lin_ee = lin_ee[:6]
            L.orc_lsc_add2(nk, nb, npair, k1.ctypes.data, k2.ctypes.data, P1ee.ctypes.data, P2ee.ctypes.data,
                           f_lin.ctypes.data, Lii.ctypes.data, Lij.ctypes.data, Lji.ctypes.data, int(antisym))
            if not fixed:
                if not antisym:
                    L.orc_lsc_add_p3p4(nb, npair, k1.ctypes.data, k2.ctypes.data, P3.ctypes.data, P4.ctypes.data,
                                       f_lin.ctypes.data, Lij.ctypes.data, Lji.ctypes.data)
                L.orc_lsc_add_p5p6(nb, npair, k1.ctypes.data, k2.ctypes.data, P5.ctypes.data, P6.ctypes.data,
                                   f_lin.ctypes.data, Lij.ctypes.data, Lji.ctypes.data)
        L.orc_lsc_diag(nb, npair, k1.ctypes.data, k2.ctypes.data, Lii.ctypes.data, Lij.ctypes.data, Lji.ctypes.data)
        P1, P2 = Lij, Lji
    ee_mode = pm.get("eeMode", "none")
    with_ee = ee_mode != "none" and not linear
    if int(pget(pm, "alg_ddmdteq", 0)) and not with_ee:
        tmp = OracleSystem(nk=nk, nb_dm=nb_dm, bstart=bstart, bend=bend, npair=npair, e_dm=e_dm, f_dm=f_dm,
                           k1st=k1, k2nd=k2, P1=np.ascontiguousarray(P1), P2=np.ascontiguousarray(P2),
                           prefac_eph=2 * math.pi / sz["nk_full"], Hcoh=None, smat=smat, dm0=dm0,
                           picture_schrodinger=schrod, expt=expt, t0=t0, tstep=0.0, tend=0.0, temperature=T, mu=mu,
                           nk_full=sz["nk_full"], ob_prefac=1.0, ode={}, params={})
        ddmdt_eq = np.zeros((nk, nb * nb), np.complex128)
        cs = tmp.cstruct()
        L.orc_compute_ddmdt_eq(C.addressof(cs), f_eq.ctypes.data, ddmdt_eq.ctypes.data)
    ee = None
    if ee_mode != "none" and not linear:  # (with alg_linearize the e-e term is part of the operators)
        if ee_mode != "Pee_update" or int(pget(pm, "alg_linearize_dPee", 0)):
            raise ValueError("the oracle restates eeMode = Pee_update without linearization")
        ee = _ee_model_of(pm, sz, dd, R, nk, nb, nb_dm, bstart, bend, e_dm, f_dm, nv_dm, T, cell_size, nfree, P1, P2)
        # set-up (ElectronPhonon.cpp:3-14): P_ee at the equilibrium occupations with the set-up density
        tmp = OracleSystem(nk=nk, nb_dm=nb_dm, bstart=bstart, bend=bend, npair=npair, e_dm=e_dm, f_dm=f_dm,
                           k1st=k1, k2nd=k2, P1=ee.P1eff, P2=ee.P2eff, prefac_eph=2 * math.pi / sz["nk_full"], Hcoh=None,
                           smat=smat, dm0=dm0, picture_schrodinger=schrod, expt=expt, t0=t0, tstep=0.0, tend=0.0,
                           temperature=T, mu=mu, nk_full=sz["nk_full"], ob_prefac=1.0, ode={}, params={})
        ee_operators(tmp, ee, None, np.ascontiguousarray(f_dm[:, bstart:bend]), nfree)
        P1, P2 = ee.P1eff, ee.P2eff
        if int(pget(pm, "alg_ddmdteq", 0)):
            # DensityMatrix_Dynamics.h:58-63: reset_scatt at rho_eq = diag(f_eq) (the screening density
            # from rho_eq when the model updates it, P_ee(rho_eq)), then compute_ddmdt_eq with those
            # operators; the rebuilds before every RHS start from there
            dm_eq = np.zeros((nk, nb_dm, nb_dm), np.complex128)
            dm_eq[:, range(nb_dm), range(nb_dm)] = f_eq
            y_eq = y_of(dm_eq.reshape(nk, -1))
            cs = tmp.cstruct()
            L.orc_ee_rebuild(C.addressof(ee.c), C.addressof(cs), C.c_double(t0), y_eq.ctypes.data)
            tmp2 = OracleSystem(nk=nk, nb_dm=nb_dm, bstart=bstart, bend=bend, npair=npair, e_dm=e_dm, f_dm=f_dm,
                                k1st=k1, k2nd=k2, P1=ee.P1eff.copy(), P2=ee.P2eff.copy(),
                                prefac_eph=2 * math.pi / sz["nk_full"], Hcoh=None, smat=smat, dm0=dm0,
                                picture_schrodinger=schrod, expt=expt, t0=t0, tstep=0.0, tend=0.0, temperature=T,
                                mu=mu, nk_full=sz["nk_full"], ob_prefac=1.0, ode={}, params={})
            ddmdt_eq = np.zeros((nk, nb * nb), np.complex128)
            cs2 = tmp2.cstruct()
            L.orc_compute_ddmdt_eq(C.addressof(cs2), f_eq.ctypes.data, ddmdt_eq.ctypes.data)
    return OracleSystem(nk=nk, nb_dm=nb_dm, bstart=bstart, bend=bend, npair=npair, e_dm=e_dm, f_dm=f_dm,
                        k1st=k1, k2nd=k2, P1=P1 if ee is not None else np.ascontiguousarray(P1),
                        P2=P2 if ee is not None else np.ascontiguousarray(P2),
                        prefac_eph=2 * math.pi / sz["nk_full"], Hcoh=Hcoh, smat=smat, dm0=dm0,
                        picture_schrodinger=schrod, expt=expt, t0=t0, tstep=tstep, tend=pget(pm, "tend", 0.0, fs),
                        temperature=T, mu=mu, nk_full=sz["nk_full"], ob_prefac=(1.0 / sz["nk_full"]) / cell_size_cmd,
                        ode=ode, params=pm, nv_dm=nv_dm, mue=mue, muh=muh, f_eq=f_eq, ddmdt_eq=ddmdt_eq, linear=linear,
                        f_lin=f_lin, ee=ee, sparse=int(pget(pm, "alg_sparseP", 0.0)) != 0,
                        lin_ee=lin_ee if linear else None,
                        thr_sparse=pget(pm, "alg_thr_sparseP", 1e-40))


def ee_operators(s: OracleSystem, ee: EEModel, dm_window, f_window, nfree):
    """P_ee of every pair (orc_ee_P) for window density matrices dm_window [nk][nb^2] (Schrodinger
    picture; dm1 = 1 - dm) or, with dm_window None, the occupations f_window [nk][nb]; then the
    system's operators P_base + scale P_ee. Returns (P1ee, P2ee)."""
    L = lib()
    cs = s.cstruct()
    if dm_window is None:
        L.orc_ee_P(C.addressof(ee.c), C.addressof(cs), None, None, f_window.ctypes.data, C.c_double(nfree),
                   ee.P1ee.ctypes.data, ee.P2ee.ctypes.data)
    else:
        dm = np.ascontiguousarray(dm_window, np.complex128)
        nb = ee.nb
        dm1 = -dm.reshape(-1, nb, nb)
        dm1[:, range(nb), range(nb)] += 1.0
        dm1 = np.ascontiguousarray(dm1.reshape(dm.shape))
        L.orc_ee_P(C.addressof(ee.c), C.addressof(cs), dm.ctypes.data, dm1.ctypes.data, None, C.c_double(nfree),
                   ee.P1ee.ctypes.data, ee.P2ee.ctypes.data)
    a1 = ee.P1ee * complex(ee.scale, 0) if ee.scale != 1.0 else ee.P1ee
    a2 = ee.P2ee * complex(ee.scale, 0) if ee.scale != 1.0 else ee.P2ee
    ee.P1eff[:] = a1 + ee.P1base
    ee.P2eff[:] = a2 + ee.P2base
    return ee.P1ee.copy(), ee.P2ee.copy()


def ee_rebuild(s: OracleSystem, t: float, y: np.ndarray):
    """reset_scatt's e-e update on state y at time t (orc_ee_rebuild): the screening density from y
    (with update_screening), P_ee(rho), P = P_base + scale P_ee. Returns (P1, P2) copies."""
    y = np.ascontiguousarray(y, dtype=np.float64)
    cs = s.cstruct()
    lib().orc_ee_rebuild(C.addressof(s.ee.c), C.addressof(cs), C.c_double(t), y.ctypes.data)
    return s.ee.P1eff.copy(), s.ee.P2eff.copy()


def set_mu_and_n(pm, e, e_dm, sz, nv_dm, T, mu, cell_size, dim):
    """electron::set_mu_and_n (electron.h:141-160) with the energy range of the electron constructor
    (electron.h:94-105). Returns mu and (carrier_bvk_gs, ne_bvk_gs, nh_bvk_gs)."""
    L = lib()
    nk, nb, nv = e.shape[0], e.shape[1], sz["nv"]
    nb_dm = e_dm.shape[1]
    big = np.finfo(np.float64).max
    sub_c = e_dm[:, nv_dm:nb_dm]
    sub_v = e_dm[:, 0:nv_dm]
    emax = float(sub_c.max()) if sub_c.size else -big
    ecmin = float(sub_c.min()) if sub_c.size else big
    evmax = float(sub_v.max()) if sub_v.size else -big
    emin = float(sub_v.min()) if sub_v.size else big
    if nb_dm == nv_dm:
        emax = evmax + 1
    if nv_dm == 0:
        emin = ecmin - 1
    cd = pget(pm, "carrier_density", 0.0, bohr2cm ** dim)
    excess = int(pget(pm, "carrier_density_means_excess_density", 0))
    nk_full = sz["nk_full"]
    ec = np.ascontiguousarray(e)
    if cd != 0 and not excess:
        mu = L.orc_find_mu_bisect(cd * nk_full * cell_size, 0, T, emin, emax, ec.ctypes.data, nk, nb, nv)
    if excess:
        mu = L.orc_find_mu_bisect(cd * nk_full * cell_size, 1, T, emin, emax, ec.ctypes.data, nk, nb, nv)
    ne = L.orc_compute_nfree(0, T, mu, ec.ctypes.data, nk, nb, nv) / nk_full / cell_size
    nh = L.orc_compute_nfree(1, T, mu, ec.ctypes.data, nk, nb, nv) / nk_full / cell_size
    nei = 0.0 / nk_full / cell_size
    nhi = 0.0 / nk_full / cell_size
    gs = (ne + nei) if abs(ne + nei) > abs(nh + nhi) else (nh + nhi)
    gs = gs * nk_full * cell_size
    return mu, (gs, ne * nk_full * cell_size, nh * nk_full * cell_size), abs(ne) + abs(nh)


def _setup_prototypes():
    L = lib()
    L.orc_dm_bpert.restype = None
    L.orc_init_dm.restype = None
    L.orc_H_BS.restype = None


def y_of(dm: np.ndarray) -> np.ndarray:
    """complex [nk][nb^2] -> interleaved double y (copy_real_from_complex, comm/ODE.h:10-15)."""
    return np.ascontiguousarray(dm).view(np.float64).reshape(-1).copy()


def rhs(s: OracleSystem, t: float, y: np.ndarray) -> np.ndarray:
    y = np.ascontiguousarray(y, dtype=np.float64)
    out = np.zeros_like(y)
    cs = s.cstruct()
    lib().orc_rhs(C.addressof(cs), t, y.ctypes.data, out.ctypes.data)
    return out


def rhs_parts(s: OracleSystem, t: float, y: np.ndarray):
    y = np.ascontiguousarray(y, dtype=np.float64)
    a = np.zeros_like(y)
    b = np.zeros_like(y)
    cs = s.cstruct()
    lib().orc_rhs_parts(C.addressof(cs), t, y.ctypes.data, a.ctypes.data, b.ctypes.data)
    return a, b


def _meas(s: OracleSystem, idir: int):
    obs = np.ascontiguousarray(s.smat[:, idir, :])
    m = _Meas(obs=obs.ctypes.data, obs_kstride=s.nb_dm * s.nb_dm, f=s.f_dm.ctypes.data, prefac=s.ob_prefac,
              bs=s.nv_dm, be=s.nb_dm)
    return m, obs


def measure(s: OracleSystem, y: np.ndarray, t: float, idir: int = 2):
    m, obs = _meas(s, idir)
    tot, amp = C.c_double(), C.c_double()
    y = np.ascontiguousarray(y, dtype=np.float64)
    lib().orc_measure(s.nk, s.nb_dm, s.nv_dm, s.nb_dm, obs.ctypes.data, s.nb_dm * s.nb_dm, s.f_dm.ctypes.data,
                      s.e_dm.ctypes.data, t, s.picture_schrodinger, y.ctypes.data, s.ob_prefac, C.byref(tot), C.byref(amp))
    return tot.value, amp.value


def rk4(s: OracleSystem, t0: float, h: float, nsteps: int, y: np.ndarray, every: int = 0, idir: int = 2):
    y = np.ascontiguousarray(y, dtype=np.float64).copy()
    nrec = nsteps // every if every > 0 else 0
    rec = np.zeros((max(nrec, 1), 3))
    m, obs = _meas(s, idir)
    cs = s.cstruct()
    lib().orc_rk4(C.addressof(cs), t0, h, nsteps, y.ctypes.data, every, C.addressof(m), rec.ctypes.data)
    return y, rec[:nrec]


def rkf45(s: OracleSystem, y: np.ndarray, t0: float, tend: float, tstep: float, hstart: float, hmin: float,
          hmax: float, epsabs: float, idir: int = 2):
    y = np.ascontiguousarray(y, dtype=np.float64).copy()
    nout = int(math.ceil((tend - t0) / tstep - 1e-9)) + 1
    rec = np.zeros((nout, 3))
    ncalls = np.zeros(nout, dtype=np.int64)
    m, obs = _meas(s, idir)
    cs = s.cstruct()
    st = lib().orc_rkf45(C.addressof(cs), t0, tend, tstep, hstart, hmin, hmax, epsabs, y.ctypes.data, C.addressof(m),
                         rec.ctypes.data, ncalls.ctypes.data, nout)
    n = int(np.count_nonzero(rec[:, 0]))
    return st, y, rec[:n], ncalls[:n]


def euler(s: OracleSystem, t0: float, h: float, nsteps: int, y: np.ndarray):
    y = np.ascontiguousarray(y, dtype=np.float64).copy()
    cs = s.cstruct()
    lib().orc_euler(C.addressof(cs), t0, h, nsteps, y.ctypes.data)
    return y


# ------------------------------------------------------------------------------------------------
# In-memory systems and the multi-process (rank-sliced) RHS used as the CPU baseline
# ------------------------------------------------------------------------------------------------
def from_arrays(*, nk, nb_dm, bstart, bend, e_dm, f_dm, k1st, k2nd, P1, P2, prefac_eph, dm0, smat=None, Hcoh=None,
                picture_schrodinger=0, expt=1, t0=0.0, temperature=0.0, mu=0.0, nk_full=1.0, ob_prefac=1.0):
    """An OracleSystem over arrays already in memory (no copies of P)."""
    return OracleSystem(nk=nk, nb_dm=nb_dm, bstart=bstart, bend=bend, npair=int(np.asarray(k1st).size),
                        e_dm=np.ascontiguousarray(e_dm, np.float64), f_dm=np.ascontiguousarray(f_dm, np.float64),
                        k1st=np.ascontiguousarray(k1st, np.uint64), k2nd=np.ascontiguousarray(k2nd, np.uint64),
                        P1=np.ascontiguousarray(P1, np.complex128), P2=np.ascontiguousarray(P2, np.complex128),
                        prefac_eph=prefac_eph, Hcoh=None if Hcoh is None else np.ascontiguousarray(Hcoh, np.complex128),
                        smat=smat, dm0=np.ascontiguousarray(dm0, np.complex128), picture_schrodinger=picture_schrodinger,
                        expt=expt, t0=t0, tstep=0.0, tend=0.0, temperature=temperature, mu=mu, nk_full=nk_full,
                        ob_prefac=ob_prefac, ode={}, params={})


_PAR = {}


def _par_worker(args):
    """One rank's pair slice; the system lives in module state inherited through fork."""
    from multiprocessing import shared_memory
    rank, p0, p1, t, names, shapes = args
    s = _PAR["sys"]
    bufs = [shared_memory.SharedMemory(name=n) for n in names]
    try:
        e_w = np.ndarray(shapes[0], np.float64, buffer=bufs[0].buf)
        dm_w = np.ndarray(shapes[1], np.complex128, buffer=bufs[1].buf)
        dm1_w = np.ndarray(shapes[1], np.complex128, buffer=bufs[2].buf)
        part = np.ndarray((shapes[2][0],) + shapes[1], np.complex128, buffer=bufs[3].buf)
        Pdm = np.zeros(shapes[1], np.complex128)
        dm1P = np.zeros(shapes[1], np.complex128)
        cs = s.cstruct()
        lib().orc_pairs_partial(C.addressof(cs), e_w.ctypes.data, t, dm_w.ctypes.data, dm1_w.ctypes.data, p0, p1,
                                Pdm.ctypes.data, dm1P.ctypes.data)
        part[2 * rank] = Pdm
        part[2 * rank + 1] = dm1P
        del e_w, dm_w, dm1_w, part
    finally:
        for b in bufs:
            b.close()
    return rank


class ParallelRHS:
    """func(t, y) evaluated as DMD does with nproc MPI ranks: contiguous pair slices
    (mymp::distribute_var, mymp.cpp:8-36), per-rank partial Pdm/dm1P, summed (the allreduce of
    evolve_eph.cpp:137), then the finish. Worker processes are forked before any GPU use and read P
    from the parent's memory."""

    def __init__(self, s: OracleSystem, nproc: int):
        import multiprocessing as mp
        from multiprocessing import shared_memory
        self.s = s
        self.nproc = max(1, int(nproc))
        nb = s.bend - s.bstart
        self.shapes = ((s.nk, nb), (s.nk, nb * nb), (2 * self.nproc,))
        sz = [s.nk * nb * 8, s.nk * nb * nb * 16, s.nk * nb * nb * 16, 2 * self.nproc * s.nk * nb * nb * 16]
        self.shm = [shared_memory.SharedMemory(create=True, size=max(z, 16)) for z in sz]
        self.e_w = np.ndarray(self.shapes[0], np.float64, buffer=self.shm[0].buf)
        self.dm_w = np.ndarray(self.shapes[1], np.complex128, buffer=self.shm[1].buf)
        self.dm1_w = np.ndarray(self.shapes[1], np.complex128, buffer=self.shm[2].buf)
        self.part = np.ndarray((2 * self.nproc,) + self.shapes[1], np.complex128, buffer=self.shm[3].buf)
        n = s.npair
        self.ranges = [((n * r) // self.nproc, (n * (r + 1)) // self.nproc) for r in range(self.nproc)]
        _PAR["sys"] = s
        self.pool = mp.get_context("fork").Pool(self.nproc) if self.nproc > 1 else None

    def __call__(self, t, y):
        s = self.s
        y = np.ascontiguousarray(y, np.float64)
        cs = s.cstruct()
        L = lib()
        L.orc_window_in(C.addressof(cs), y.ctypes.data, self.e_w.ctypes.data, self.dm_w.ctypes.data,
                        self.dm1_w.ctypes.data)
        jobs = [(r, p0, p1, float(t), [m.name for m in self.shm], self.shapes) for r, (p0, p1) in enumerate(self.ranges)]
        if self.pool is not None:
            list(self.pool.map(_par_worker, jobs))
        else:
            _par_worker(jobs[0])
        Pdm = self.part[0::2].sum(axis=0)
        dm1P = self.part[1::2].sum(axis=0)
        out = np.zeros_like(y)
        L.orc_rhs_from_partials(C.addressof(cs), float(t), y.ctypes.data, self.e_w.ctypes.data, self.dm_w.ctypes.data,
                                self.dm1_w.ctypes.data, Pdm.ctypes.data, dm1P.ctypes.data, out.ctypes.data)
        return out

    def close(self):
        if self.pool is not None:
            self.pool.terminate()
            self.pool = None
        for a in ("e_w", "dm_w", "dm1_w", "part"):
            setattr(self, a, None)
        for m in self.shm:
            m.close()
            m.unlink()
        self.shm = []
