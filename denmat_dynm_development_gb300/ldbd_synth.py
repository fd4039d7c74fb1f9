"""Seeded synthetic ``ldbd_data`` generator.

Writes exactly the binary/text files that DMD's readers consume, so the same directory can be
fed to the reference program and to this package:

* ``ldbd_size.dat`` -- text header read by ``electron::read_ldbd_size`` (electron.cpp:100-133),
  ``electronphonon::get_brange/get_nkpair`` (ElectronPhonon.cpp:132-177), ``phonon::read_jdftx``
  (phonon.h:49-79) and ``parameters::read_jdftx`` (parameters.cpp:7-23).
* ``ldbd_R.dat`` -- dimension + lattice vectors (lattice.h:48-56).
* ``ldbd_kvec.bin`` double[nk][3], ``ldbd_ek.bin`` double[nk][nb], ``ldbd_smat.bin``
  complex128[nk][3][nb*nb] (electron.cpp:134-314).
* optionally ``ldbd_Umat.bin`` complex128[nk][nb_wannier][nb_eph] (electron.cpp:388-410): the
  e-ph window's columns of the Wannier rotations, whose overlaps U_k^dag U_k' enter the e-e model
  (ElecElec_Model.h:72-79). The reader's full-matrix branch depends on a size check that returns
  no value when the sizes match (comm/myio.cpp:133-137), so only this partial layout loads reliably.
* ``ldbd_kpair_k1st.bin`` / ``ldbd_kpair_k2nd.bin`` uint64[npair] with k1st <= k2nd
  (ElectronPhonon.cpp:182-204).
* ``ldbd_P1_lindblad.bin`` / ``ldbd_P2_lindblad.bin`` complex128[npair][nb^4], row-major
  ``[(i1*nb+i2)*nb*nb + i3*nb + i4]`` (ElectronPhonon.cpp:209-253).
* optionally ``ldbd_P1_lindblad_D1.bin`` / ``ldbd_P2_lindblad_D1.bin`` -- the ab-initio
  ("ab_neutral") electron-impurity operators that DMD scales by |n_i V_cell| and adds into P
  (ElectronImpurity.cpp:3-49).

The P operators follow the Lindblad initializer's construction
(lindbladInit_for-DMD-4.5.6/ElectronPhonon.h:432-572): per phonon mode and for emission /
absorption, G = g * sqrt(prefac_delta * exp(-(dE +- w)^2 / (2 sigma^2))) inside the energy cutoff,
A = G*sqrt(n_q+1) or G*sqrt(n_q), and

    P1[(i1 i2),(i3 i4)] += App[i1,i3] conj(App[i2,i4]) + Amm[i1,i3] conj(Amm[i2,i4])
    P2[(i1 i2),(i3 i4)] += Amp[i3,i1] conj(Amp[i4,i2]) + Apm[i3,i1] conj(Apm[i4,i2])

The electron-impurity operator is the elastic analogue with a single A (ElecImp_Model.h:185-214).
Random numbers come from ``numpy.random.default_rng([seed, stream, chunk])`` so any chunk can be
regenerated on its own.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field, asdict
from typing import Optional, Sequence

import numpy as np

from . import units


@dataclass
class SynthConfig:
    nk: int = 500                    # k-points kept
    nb: int = 2                      # bands (2: spin-split pair, 4: two spin-split pairs)
    seed: int = 0
    meff: float = 0.3                # parabolic-band effective mass (electron masses)
    ewindow_ev: float = 0.2          # energy window above the band bottom
    split_mev: float = 2.0           # spin splitting Delta ~ U(0, split)
    pair_offset_mev: float = 50.0    # nb=4: offset of the second spin pair
    de_pair_mev: float = 60.0        # k-pairs kept when |E_k - E_k'| < de_pair
    nmodes: int = 6
    omega_mev: Sequence[float] = (5.0, 60.0)
    g_sigma_mev: float = 20.0
    degauss_mev: float = 10.0
    ndegauss: float = 5.0
    temperature_K: float = 300.0
    mu_below_cbm_ev: float = 0.1     # chemical potential below the band bottom
    spin_mix: float = 0.1            # spin-mixing angle scale of the band eigenvectors
    lattice_a_bohr: float = 10.68    # fcc lattice constant
    eimp_sigma_mev: Optional[float] = None   # write D1 e-imp files when set
    ecbm_ha: float = 0.05            # absolute energy of the band bottom (Ha)
    extra_bands: int = 0             # bands of the density matrix below the e-ph window
    nv: int = 0                      # lowest bands declared valence in ldbd_size.dat (holes)
    nwannier: Optional[int] = None   # write ldbd_Umat.bin with this many Wannier functions (>= nb_dm)
    kball: bool = False              # keep the nk lowest-energy grid points (a ball: k1 + k3 - k2 mostly inside)
    chunk_pairs: int = 1 << 18

    def to_dict(self):
        return asdict(self)


@dataclass
class SynthInfo:
    nk: int
    nb: int
    npair: int
    nk_full: float
    kmesh: tuple
    cell_volume: float
    temperature: float
    mu: float
    mode_omega: list = field(default_factory=list)


def _fcc(a):
    return 0.5 * a * np.array([[0.0, 1.0, 1.0], [1.0, 0.0, 1.0], [1.0, 1.0, 0.0]])


def _kset(cfg: SynthConfig, rng):
    """Grid k-points (fractional) inside the energy window, randomly subsampled to nk."""
    R = _fcc(cfg.lattice_a_bohr)
    V = abs(np.linalg.det(R))
    B = 2.0 * np.pi * np.linalg.inv(R).T          # k_cart = B @ k_frac
    emax = cfg.ewindow_ev * units.eV
    kmax = math.sqrt(2.0 * cfg.meff * emax)
    vbz = (2.0 * np.pi) ** 3 / V
    sphere = 4.0 / 3.0 * np.pi * kmax ** 3
    n = int(math.ceil((1.4 * cfg.nk * vbz / sphere) ** (1.0 / 3.0)))
    n = max(n, 4)
    binv = np.linalg.norm(np.linalg.inv(B), 2)
    while True:
        M = int(math.ceil(n * binv * kmax)) + 1
        r = np.arange(-M, M + 1)
        g = np.stack(np.meshgrid(r, r, r, indexing="ij"), -1).reshape(-1, 3)
        kf = g / float(n)
        kc = kf @ B.T
        e = (kc ** 2).sum(1) / (2.0 * cfg.meff)
        keep = np.nonzero(e < emax)[0]
        if keep.size >= int(1.2 * cfg.nk) + 1:
            break
        n += 1
    if cfg.kball:
        sel = np.sort(keep[np.argsort(e[keep], kind="stable")[:cfg.nk]])
    else:
        sel = np.sort(rng.choice(keep, size=cfg.nk, replace=False))
    rng.shuffle(sel)                       # a random k order, as a k-point selection would give
    return R, V, n, kf[sel], e[sel]


def _bands(cfg: SynthConfig, e0, rng):
    nk = e0.size
    d1 = rng.uniform(0.0, cfg.split_mev * 1e-3 * units.eV, nk)
    if cfg.nb == 2:
        e = np.stack([e0 - 0.5 * d1, e0 + 0.5 * d1], 1)
    elif cfg.nb == 4:
        d2 = rng.uniform(0.0, cfg.split_mev * 1e-3 * units.eV, nk)
        off = cfg.pair_offset_mev * 1e-3 * units.eV
        e = np.stack([e0 - 0.5 * d1, e0 + 0.5 * d1, e0 + off - 0.5 * d2, e0 + off + 0.5 * d2], 1)
    else:
        raise ValueError("nb must be 2 or 4")
    if cfg.extra_bands:
        lo = np.stack([e[:, 0] - (cfg.extra_bands - i) * 0.02 * units.eV for i in range(cfg.extra_bands)], 1)
        e = np.concatenate([lo, e], 1)
    return e + cfg.ecbm_ha


def _spin(cfg: SynthConfig, nk, rng):
    """S_d(k) = 1/2 U_k^dag Sigma_d U_k with U_k = exp(i * mix * H_k), H_k random Hermitian."""
    nb = cfg.nb + cfg.extra_bands
    sig = np.array([[[0, 1], [1, 0]], [[0, -1j], [1j, 0]], [[1, 0], [0, -1]]], dtype=np.complex128)
    if nb % 2 == 0 and nb > 2:
        sig = np.stack([np.kron(np.eye(nb // 2), s) for s in sig])
    a = rng.standard_normal((nk, nb, nb)) + 1j * rng.standard_normal((nk, nb, nb))
    h = 0.5 * (a + np.conj(np.swapaxes(a, 1, 2))) / math.sqrt(2.0 * nb)
    w, v = np.linalg.eigh(h)
    u = np.einsum("kij,kj,klj->kil", v, np.exp(1j * cfg.spin_mix * w), np.conj(v))
    ud = np.conj(np.swapaxes(u, 1, 2))
    s = 0.5 * np.einsum("kij,djl,klm->kdim", ud, sig, u)
    s = 0.5 * (s + np.conj(np.swapaxes(s, 2, 3)))   # exactly Hermitian
    return s.reshape(nk, 3, nb * nb)


def _pairs(cfg: SynthConfig, e):
    """All (k, k') with k <= k' and |Ebar_k - Ebar_k'| < de_pair, in k-major order."""
    ebar = e.mean(1)
    order = np.argsort(ebar, kind="stable")
    es = ebar[order]
    w = cfg.de_pair_mev * 1e-3 * units.eV
    lo = np.searchsorted(es, ebar - w, side="right")
    hi = np.searchsorted(es, ebar + w, side="left")
    k1, k2 = [], []
    for ik in range(e.shape[0]):
        cand = order[lo[ik]:hi[ik]]
        cand = np.sort(cand[cand >= ik])
        cand = cand[np.abs(ebar[cand] - ebar[ik]) < w]
        k1.append(np.full(cand.size, ik, dtype=np.uint64))
        k2.append(cand.astype(np.uint64))
    return np.concatenate(k1), np.concatenate(k2)


def _cgauss(rng, shape, sigma):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) * (sigma / math.sqrt(2.0))


def _sum_outer(A, transpose):
    """sum_m A_m[i1,i3] conj(A_m[i2,i4]) (P1 form) or sum_m A_m[i3,i1] conj(A_m[i4,i2]) (P2 form),
    returned as [n][(i1*nb+i2)*nb*nb + i3*nb + i4]. A has shape (n, m, nb, nb)."""
    n, m, nb, _ = A.shape
    if transpose:
        A = np.swapaxes(A, 2, 3)
    X = A.reshape(n, m, nb * nb)                       # [n][m][(i1 i3)]
    M = np.matmul(np.swapaxes(X, 1, 2), np.conj(X))    # [n][(i1 i3)][(i2 i4)]
    return np.ascontiguousarray(M.reshape(n, nb, nb, nb, nb).transpose(0, 1, 3, 2, 4)).reshape(n, nb ** 4)


def eph_chunk(cfg: SynthConfig, ek, ekp, omegas, chunk_index):
    """P1, P2 (complex128 [n][nb^4]) of the e-ph term for one chunk of pairs."""
    A1, A2 = eph_amplitudes(cfg, ek, ekp, omegas, chunk_index)
    return _sum_outer(A1, False), _sum_outer(A2, True)


def eph_chunk_modes(cfg: SynthConfig, ek, ekp, omegas, chunk_index):
    """The e-ph P1, P2 of one chunk split by phonon mode: [nmodes][n][nb^4] each (their sum over modes
    is eph_chunk's, up to rounding). A scale on mode m's coupling |g|^2 scales its operators."""
    A1, A2 = eph_amplitudes(cfg, ek, ekp, omegas, chunk_index)
    nm = len(omegas)
    return (np.stack([_sum_outer(A1[:, 2 * m:2 * m + 2], False) for m in range(nm)]),
            np.stack([_sum_outer(A2[:, 2 * m:2 * m + 2], True) for m in range(nm)]))


def eph_amplitudes(cfg: SynthConfig, ek, ekp, omegas, chunk_index):
    """Emission/absorption amplitudes per mode: A1 = (App, Amm), A2 = (Amp, Apm) per mode, [n][2 nmodes][nb][nb]."""
    rng = np.random.default_rng([cfg.seed, 1, chunk_index])
    n, nb = ek.shape
    T = cfg.temperature_K * units.Kelvin
    sigma = cfg.degauss_mev * 1e-3 * units.eV
    ethr = sigma * cfg.ndegauss
    gsig = cfg.g_sigma_mev * 1e-3 * units.eV
    sq_delta = math.sqrt(1.0 / (sigma * math.sqrt(2.0 * math.pi)))
    dE = ek[:, :, None] - ekp[:, None, :]
    nm = len(omegas)
    A1 = np.empty((n, 2 * nm, nb, nb), np.complex128)   # App, Amm per mode (P1 terms)
    A2 = np.empty((n, 2 * nm, nb, nb), np.complex128)   # Amp, Apm per mode (P2 terms)
    for im, w in enumerate(omegas):
        nq = 1.0 / math.expm1(max(1e-3, w / T))
        gp = _cgauss(rng, (n, nb, nb), gsig)
        gm = _cgauss(rng, (n, nb, nb), gsig)
        xp = dE + w
        xm = dE - w
        G2p = np.where(np.abs(xp) < ethr, sq_delta * gp * np.exp(-xp * xp / (4.0 * sigma * sigma)), 0)
        G2m = np.where(np.abs(xm) < ethr, sq_delta * gm * np.exp(-xm * xm / (4.0 * sigma * sigma)), 0)
        A1[:, 2 * im] = G2p * math.sqrt(nq + 1.0)       # App
        A1[:, 2 * im + 1] = G2m * math.sqrt(nq)         # Amm
        A2[:, 2 * im] = G2m * math.sqrt(nq + 1.0)       # Amp
        A2[:, 2 * im + 1] = G2p * math.sqrt(nq)         # Apm
    return A1, A2


def eimp_chunk(cfg: SynthConfig, ek, ekp, chunk_index):
    """Elastic e-imp P1, P2 (unscaled) for one chunk of pairs."""
    rng = np.random.default_rng([cfg.seed, 2, chunk_index])
    n, nb = ek.shape
    sigma = cfg.degauss_mev * 1e-3 * units.eV
    ethr = sigma * cfg.ndegauss
    gsig = cfg.eimp_sigma_mev * 1e-3 * units.eV
    sq_delta = math.sqrt(1.0 / (sigma * math.sqrt(2.0 * math.pi)))
    dE = ek[:, :, None] - ekp[:, None, :]
    g = _cgauss(rng, (n, nb, nb), gsig)
    A = np.where(np.abs(dE) < ethr, sq_delta * g * np.exp(-dE * dE / (4.0 * sigma * sigma)), 0)[:, None]
    return _sum_outer(A, False), _sum_outer(A, True)


def umat(cfg: SynthConfig, kf):
    """Wannier rotations U_k = exp(i (H0 + sum_d k_d A_d)), [nk][nbw][nbw] unitary and smooth in the
    fractional k (H0, A_d fixed random Hermitian), so that overlaps of nearby k are near identity."""
    nbw = cfg.nwannier
    rng = np.random.default_rng([cfg.seed, 4])

    def herm():
        a = rng.standard_normal((nbw, nbw)) + 1j * rng.standard_normal((nbw, nbw))
        return 0.5 * (a + a.conj().T) / math.sqrt(2.0 * nbw)

    H0 = herm()
    A = np.stack([herm() for _ in range(3)])
    h = H0[None] + 4.0 * np.einsum("kd,dij->kij", kf, A)
    w, v = np.linalg.eigh(h)
    return np.einsum("kij,kj,klj->kil", v, np.exp(1j * w), np.conj(v))


def mode_energies(cfg: SynthConfig):
    rng = np.random.default_rng([cfg.seed, 3])
    lo, hi = cfg.omega_mev
    return list(rng.uniform(lo, hi, cfg.nmodes) * 1e-3 * units.eV)


@dataclass
class SynthSetup:
    cfg: SynthConfig
    R: np.ndarray
    V: float
    n: int
    kf: np.ndarray
    e: np.ndarray          # [nk][nb_dm] all density-matrix bands
    ew: np.ndarray         # [nk][nb] e-ph window
    s: np.ndarray          # [nk][3][nb_dm^2]
    k1: np.ndarray
    k2: np.ndarray
    omegas: list
    T: float
    mu: float

    @property
    def npair(self):
        return int(self.k1.size)

    def info(self):
        return SynthInfo(nk=self.cfg.nk, nb=self.cfg.nb, npair=self.npair, nk_full=float(self.n) ** 3,
                         kmesh=(self.n, self.n, self.n), cell_volume=self.V, temperature=self.T, mu=self.mu,
                         mode_omega=self.omegas)

    def chunk_size(self):
        return self.cfg.chunk_pairs if self.cfg.nb == 2 else max(1, self.cfg.chunk_pairs // 8)


def setup(cfg: SynthConfig) -> SynthSetup:
    """k-points, bands, spin matrices, k-pairs and mode energies of a synthetic system."""
    rng = np.random.default_rng([cfg.seed, 0])
    R, V, n, kf, e0 = _kset(cfg, rng)
    e = _bands(cfg, e0, rng)
    s = _spin(cfg, cfg.nk, rng)
    ew = np.ascontiguousarray(e[:, cfg.extra_bands:])
    k1, k2 = _pairs(cfg, ew)
    return SynthSetup(cfg=cfg, R=R, V=V, n=n, kf=kf, e=e, ew=ew, s=s, k1=k1, k2=k2, omegas=mode_energies(cfg),
                      T=cfg.temperature_K * units.Kelvin, mu=ew.min() - cfg.mu_below_cbm_ev * units.eV)


def _chunk(st: SynthSetup, ic: int):
    C = st.chunk_size()
    p0 = ic * C
    p1 = min(st.npair, p0 + C)
    ek = st.ew[st.k1[p0:p1].astype(np.int64)]
    ekp = st.ew[st.k2[p0:p1].astype(np.int64)]
    P1, P2 = eph_chunk(st.cfg, ek, ekp, st.omegas, ic)
    Q = eimp_chunk(st.cfg, ek, ekp, ic) if st.cfg.eimp_sigma_mev is not None else None
    return p0, p1, P1, P2, Q


def pair_chunks(st: SynthSetup, threads: int = 1):
    """Yield (p0, p1, P1, P2, (Q1, Q2) or None) in pair order, computed by a thread pool."""
    nch = (st.npair + st.chunk_size() - 1) // st.chunk_size()
    if threads <= 1:
        for ic in range(nch):
            yield _chunk(st, ic)
        return
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=threads) as ex:
        futs = {}
        nxt = 0
        for ic in range(nch):
            while nxt < nch and nxt < ic + 2 * threads:
                futs[nxt] = ex.submit(_chunk, st, nxt)
                nxt += 1
            yield futs.pop(ic).result()


def _proc_chunk(args):
    """Worker: one chunk of pairs written into shared memory (spawned process, numpy only)."""
    from multiprocessing import shared_memory
    cfg_d, ew, k1, k2, omegas, ic, p0, names, nb4, npair, fold = args
    cfg = SynthConfig(**cfg_d)
    ek = ew[k1.astype(np.int64)]
    ekp = ew[k2.astype(np.int64)]
    P1, P2 = eph_chunk(cfg, ek, ekp, omegas, ic)
    Q = eimp_chunk(cfg, ek, ekp, ic) if cfg.eimp_sigma_mev is not None else None
    if Q is not None and fold is not None:
        P1 = P1 + Q[0] * fold
        P2 = P2 + Q[1] * fold
    outs = [P1, P2] + ([Q[0], Q[1]] if (Q is not None and fold is None) else [])
    p1 = p0 + P1.shape[0]
    for name, arr in zip(names, outs):
        shm = shared_memory.SharedMemory(name=name)
        try:
            view = np.ndarray((npair, nb4), np.complex128, buffer=shm.buf)
            view[p0:p1] = arr
            del view
        finally:
            shm.close()
    return ic


def generate_arrays(cfg: SynthConfig, fold_fraction: Optional[float] = None, procs: Optional[int] = None):
    """All arrays of a synthetic system in memory. With fold_fraction the e-imp operators are folded
    into P as DMD does at set-up (P += fraction * P_D1); otherwise they are returned separately.
    Chunks are computed by `procs` spawned worker processes into shared memory; the result does not
    depend on the number of processes."""
    st = setup(cfg)
    procs = procs or min(16, os.cpu_count() or 1)
    nb4 = cfg.nb ** 4
    npair = st.npair
    want_q = cfg.eimp_sigma_mev is not None and fold_fraction is None
    if procs <= 1 or npair <= st.chunk_size():
        P1 = np.empty((npair, nb4), np.complex128)
        P2 = np.empty((npair, nb4), np.complex128)
        Q1 = np.empty((npair, nb4), np.complex128) if want_q else None
        Q2 = np.empty((npair, nb4), np.complex128) if want_q else None
        for p0, p1, a1, a2, Q in pair_chunks(st, 1):
            if Q is not None and fold_fraction is not None:
                a1 = a1 + Q[0] * fold_fraction
                a2 = a2 + Q[1] * fold_fraction
            P1[p0:p1] = a1
            P2[p0:p1] = a2
            if want_q:
                Q1[p0:p1] = Q[0]
                Q2[p0:p1] = Q[1]
        return st, P1, P2, Q1, Q2
    import multiprocessing as mp
    from multiprocessing import shared_memory
    nbytes = npair * nb4 * 16
    shms = [shared_memory.SharedMemory(create=True, size=max(nbytes, 1)) for _ in range(4 if want_q else 2)]
    try:
        C = st.chunk_size()
        jobs = []
        for ic, p0 in enumerate(range(0, npair, C)):
            p1 = min(npair, p0 + C)
            jobs.append((cfg.to_dict(), st.ew, st.k1[p0:p1], st.k2[p0:p1], st.omegas, ic, p0,
                         [m.name for m in shms], nb4, npair, fold_fraction))
        with mp.get_context("spawn").Pool(processes=procs) as pool:
            for _ in pool.imap_unordered(_proc_chunk, jobs):
                pass
        outs = []
        for m in shms:
            outs.append(np.ndarray((npair, nb4), np.complex128, buffer=m.buf).copy())
    finally:
        for m in shms:
            m.close()
            m.unlink()
    return (st, outs[0], outs[1], outs[2] if want_q else None, outs[3] if want_q else None)


def _modes_worker(args):
    """Worker (spawned process, numpy only): one chunk of the per-parameter operator sets (the phonon
    modes, then the unscaled e-imp operators when the configuration has them) put to one use:
      ("scaled", theta): P = sum_m theta_m P^(m) written to the two output buffers;
      ("mode", m):       P^(m) written to the two output buffers;
      ("contract", _):   Re sum conj(G) P^(m) for every m, with G read from the two buffers."""
    from multiprocessing import shared_memory
    cfg_d, ew, k1, k2, omegas, ic, p0, names, nb4, npair, job = args
    cfg = SynthConfig(**cfg_d)
    ek = ew[k1.astype(np.int64)]
    ekp = ew[k2.astype(np.int64)]
    a1, a2 = eph_chunk_modes(cfg, ek, ekp, omegas, ic)
    if cfg.eimp_sigma_mev is not None:
        q1, q2 = eimp_chunk(cfg, ek, ekp, ic)
        a1 = np.concatenate([a1, q1[None]])
        a2 = np.concatenate([a2, q2[None]])
    p1 = p0 + a1.shape[1]
    bufs = [shared_memory.SharedMemory(name=n) for n in names]
    try:
        views = np.ndarray((2, npair, nb4), np.complex128, buffer=bufs[0].buf)
        kind, arg = job
        out = None
        if kind == "scaled":
            th = np.asarray(arg, np.float64)
            views[0][p0:p1] = np.tensordot(th, a1, 1)
            views[1][p0:p1] = np.tensordot(th, a2, 1)
        elif kind == "mode":
            views[0][p0:p1] = a1[arg]
            views[1][p0:p1] = a2[arg]
        else:
            g1, g2 = views[0][p0:p1], views[1][p0:p1]
            out = np.array([np.vdot(g1, a1[m]).real + np.vdot(g2, a2[m]).real for m in range(a1.shape[0])])
        del views
    finally:
        for b in bufs:
            b.close()
    return ic, out


class SharedPair:
    """complex128 [2][npair][nb^4] in shared memory -- the operators P1, P2 or a gradient with respect
    to them, one block after the other as the library's dJdP -- readable by the generator's worker
    processes; a[0], a[1] are the two blocks; close() releases them."""

    def __init__(self, npair, nb4):
        from multiprocessing import shared_memory
        self.shm = [shared_memory.SharedMemory(create=True, size=max(16, 2 * npair * nb4 * 16))]
        self.a = np.ndarray((2, npair, nb4), np.complex128, buffer=self.shm[0].buf)

    def close(self):
        self.a = None
        for m in self.shm:
            m.close()
            m.unlink()
        self.shm = []


class ModeSets:
    """The per-parameter operator sets of a synthetic system (the phonon modes' |g|^2 scales, then the
    impurity operator when cfg.eimp_sigma_mev is set), produced chunk by chunk by `procs` spawned
    worker processes and never held together: P(theta) = sum_m theta_m P^(m), one set P^(m), or the
    contractions Re sum conj(G) P^(m) with a gradient G. The chunks are the generator's, so every
    set equals mode_operators' arrays."""

    def __init__(self, cfg: SynthConfig, procs: Optional[int] = None):
        self.cfg = cfg
        self.st = setup(cfg)
        self.procs = procs or min(16, os.cpu_count() or 1)
        self.nb4 = cfg.nb ** 4
        self.nparams = cfg.nmodes + (1 if cfg.eimp_sigma_mev is not None else 0)

    def _run(self, pair: SharedPair, job):
        import multiprocessing as mp
        st, C = self.st, self.st.chunk_size()
        jobs = [(self.cfg.to_dict(), st.ew, st.k1[p0:min(st.npair, p0 + C)], st.k2[p0:min(st.npair, p0 + C)],
                 st.omegas, ic, p0, [m.name for m in pair.shm], self.nb4, st.npair, job)
                for ic, p0 in enumerate(range(0, st.npair, C))]
        with mp.get_context("spawn").Pool(processes=self.procs) as pool:
            return [r for _, r in sorted(pool.imap_unordered(_modes_worker, jobs), key=lambda x: x[0])]

    def scaled(self, theta) -> SharedPair:
        out = SharedPair(self.st.npair, self.nb4)
        self._run(out, ("scaled", [float(x) for x in theta]))
        return out

    def mode(self, m: int) -> SharedPair:
        out = SharedPair(self.st.npair, self.nb4)
        self._run(out, ("mode", int(m)))
        return out

    def contract(self, G: SharedPair) -> np.ndarray:
        return np.sum(self._run(G, ("contract", None)), axis=0)


def mode_operators(cfg: SynthConfig):
    """Per-mode e-ph operators and the unscaled e-imp operators of a (small) synthetic system:
    (setup, P1m [nmodes][npair][nb^4], P2m, Q1 or None, Q2 or None), chunk by chunk in one process."""
    st = setup(cfg)
    nb4, nm = cfg.nb ** 4, cfg.nmodes
    P1m = np.empty((nm, st.npair, nb4), np.complex128)
    P2m = np.empty((nm, st.npair, nb4), np.complex128)
    want_q = cfg.eimp_sigma_mev is not None
    Q1 = np.empty((st.npair, nb4), np.complex128) if want_q else None
    Q2 = np.empty((st.npair, nb4), np.complex128) if want_q else None
    C = st.chunk_size()
    for ic, p0 in enumerate(range(0, st.npair, C)):
        p1 = min(st.npair, p0 + C)
        ek = st.ew[st.k1[p0:p1].astype(np.int64)]
        ekp = st.ew[st.k2[p0:p1].astype(np.int64)]
        a1, a2 = eph_chunk_modes(cfg, ek, ekp, st.omegas, ic)
        P1m[:, p0:p1] = a1
        P2m[:, p0:p1] = a2
        if want_q:
            Q1[p0:p1], Q2[p0:p1] = eimp_chunk(cfg, ek, ekp, ic)
    return st, P1m, P2m, Q1, Q2


def make_ldbd(outdir: str, cfg: SynthConfig, write_param: bool = True, threads: int = 1, **param_kw) -> SynthInfo:
    """Write ``outdir/ldbd_data/*`` (and ``outdir/param.in``) for ``cfg``."""
    d = os.path.join(outdir, "ldbd_data")
    os.makedirs(d, exist_ok=True)
    st = setup(cfg)
    e, R, n, nb, nx = st.e, st.R, st.n, cfg.nb, cfg.extra_bands
    ndm = nb + nx
    nbw = cfg.nwannier or ndm
    if nbw < ndm:
        raise ValueError("nwannier must be >= the density-matrix bands")
    mu, T = st.mu, st.T
    with open(os.path.join(d, "ldbd_size.dat"), "w") as f:
        f.write("There are scatterings only for conduction electrons\n")
        f.write("%d %d 0 %d %d %d %d 0 0 # nb nv bBot_dm bTop_dm bBot_eph_elec bTop_eph_elec nb_wannier bBot_probe band_dft_skipped\n"
                % (ndm, cfg.nv, ndm, nx, ndm, nbw))
        f.write("%21.14le %d %d %d %d # nk_full nk kmesh\n" % (float(n) ** 3, cfg.nk, n, n, n))
        f.write("%d # nkpair_elec\n" % st.npair)
        f.write("0 %d 0 0# modeStart modeStp modeSkipStart modeSkipStop\n" % cfg.nmodes)
        f.write("%21.14le # T\n" % T)
        f.write("%21.14le %21.14le %21.14le # muMin, muMax mu (given carrier density)\n" % (mu, mu, mu))
        f.write("%.17g %.17g # degauss\n" % (cfg.degauss_mev * 1e-3 * units.eV, cfg.ndegauss))
        f.write("%14.7le %14.7le %14.7le %14.7le %14.7le %14.7le # EBot_probe, ETop_probe, EBot_dm, ETop_dm, EBot_eph, ETop_eph\n"
                % (e.min(), e.max(), e.min(), e.max(), e.min(), e.max()))
        f.write("%14.7le # omegaMax" % max(st.omegas))
    with open(os.path.join(d, "ldbd_R.dat"), "w") as f:
        f.write("3\n")
        for i in range(3):
            f.write("%.17g %.17g %.17g\n" % tuple(R[i]))
    st.kf.astype(np.float64).tofile(os.path.join(d, "ldbd_kvec.bin"))
    if cfg.nwannier:
        U = umat(cfg, st.kf)[:, :, nx:nx + nb]
        np.ascontiguousarray(U, np.complex128).tofile(os.path.join(d, "ldbd_Umat.bin"))
    e.astype(np.float64).tofile(os.path.join(d, "ldbd_ek.bin"))
    st.s.astype(np.complex128).tofile(os.path.join(d, "ldbd_smat.bin"))
    st.k1.tofile(os.path.join(d, "ldbd_kpair_k1st.bin"))
    st.k2.tofile(os.path.join(d, "ldbd_kpair_k2nd.bin"))
    names = [("ldbd_P1_lindblad.bin", "ldbd_P2_lindblad.bin")]
    if cfg.eimp_sigma_mev is not None:
        names.append(("ldbd_P1_lindblad_D1.bin", "ldbd_P2_lindblad_D1.bin"))
    files = [(open(os.path.join(d, a), "wb"), open(os.path.join(d, b), "wb")) for a, b in names]
    try:
        for p0, p1, P1, P2, Q in pair_chunks(st, threads):
            files[0][0].write(P1.tobytes())
            files[0][1].write(P2.tobytes())
            if Q is not None:
                files[1][0].write(Q[0].tobytes())
                files[1][1].write(Q[1].tobytes())
    finally:
        for a, b in files:
            a.close()
            b.close()
    info = st.info()
    if write_param:
        write_param_in(outdir, cfg, info, **param_kw)
    return info


def write_param_in(outdir: str, cfg: SynthConfig, info: SynthInfo, *, tstep_fs=1.0, tend_fs=10.0,
                   Bpert_T=(0.0, 0.0, 0.1), B_T=(0.0, 0.0, 0.0), eimp_fraction=1e-4,
                   ode_method="rkf45", extra: Optional[dict] = None):
    """param.in with the keys DMD's ``parameters::read_param`` (parameters.cpp:48-529) reads."""
    lines = [
        "restart = 0",
        "code = jdftx",
        "alg_eph_sepr_eh = 1",
        "alg_eph_need_elec = 1",
        "alg_eph_need_hole = 0",
        "alg_scatt = lindblad",
        "need_imsig = 0",
        "Bxpert = %.17g" % Bpert_T[0],
        "Bypert = %.17g" % Bpert_T[1],
        "Bzpert = %.17g" % Bpert_T[2],
        "t0 = 0",
        "tend = %.17g" % tend_fs,
        "tstep = %.17g" % tstep_fs,
        "freq_measure_ene = 1000000000",
        "freq_compute_tau = 1000000000",
        "alg_ode_method = %s" % ode_method,
    ]
    if any(abs(b) > 0 for b in B_T):
        lines += ["Bx = %.17g" % B_T[0], "By = %.17g" % B_T[1], "Bz = %.17g" % B_T[2]]
    if cfg.eimp_sigma_mev is not None:
        # DMD scales the D1 operators by fraction = |n_i * V_cell| (ElectronImpurity.h:18);
        # impurity_density is read in cm^-3 and converted with bohr2cm^3 (parameters.cpp:221).
        ni_au = eimp_fraction / info.cell_volume
        lines += ["impurity_density = %.17g" % (ni_au / units.bohr2cm ** 3), "impMode = ab_neutral"]
    for k, v in (extra or {}).items():
        lines.append("%s = %s" % (k, v))
    with open(os.path.join(outdir, "param.in"), "w") as f:
        f.write("\n".join(lines) + "\n")


# Workloads named by what they are, with their sizes.
WORKLOADS = {
    # Si-like plain FP64 case: nb=2, nk=500, ~50k pairs.
    "si_nk500": SynthConfig(nk=500, nb=2, de_pair_mev=60.0),
    # GaAs-like at scale: nb=2, nk=20k, ~10M pairs, e-ph + e-imp.
    "gaas_nk20k": SynthConfig(nk=20000, nb=2, de_pair_mev=4.45, eimp_sigma_mev=5.0),
    # the same generator at nk=16k (~6.2M pairs, P 3.2 GB): profiling case with several waves of work
    "gaas_nk16k": SynthConfig(nk=16000, nb=2, de_pair_mev=4.45, eimp_sigma_mev=5.0),
    # the same generator at nk=8k (~1.6M pairs, P 0.8 GB): profiling-sized GaAs-like case
    "gaas_nk8k": SynthConfig(nk=8000, nb=2, de_pair_mev=4.45, eimp_sigma_mev=5.0),
    # MoS2-like precision case: nb=4 (two spin-split pairs), nk=30k, 4.19M pairs (P 34 GB complex128).
    "mos2_nk30k": SynthConfig(nk=30000, nb=4, de_pair_mev=0.8),
    # the same nb=4 generator at nk=2000 (~46k pairs): T1 comparisons of the nb=4 forms
    "mos2_nk2k": SynthConfig(nk=2000, nb=4, de_pair_mev=0.8),
}
