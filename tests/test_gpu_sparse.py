"""The sparse contraction (DMD_FLAG_SPARSE: alg_sparseP / alg_Pin_is_sparse) against the reference.

The golden cases nb4_sparse and nb2_sparse were made by the reference's own sparse branch
(alg_sparseP = 1: sparse_mat per pair, compute_sPt, sparse_zgemm; evolve_eph.cpp:67-82) on operators
with structural zeros; the oracle restates that branch bit for bit (test_oracle_golden). The GPU's
sparse form is held to the FP64 bounds of the dense forms: RHS 1e-12 normwise, 40 RK4 steps 1e-10,
DMD's RKF45 loop with the same RHS-call counts. Edge cases: dense operators given to the sparse form,
the additive (e-imp) operators folded before the elements are filtered, DMD's sparse operator files,
nb = 1 and 3 windows, an empty pair list, a state that is not Hermitian.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from test_gpu_parity import _random_system, rel, write_sparse

pytestmark = pytest.mark.gpu

SPARSE_CASES = ["nb4_sparse", "nb2_sparse"]


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as G
    G.build()


def make_sparse(s, **kw):
    from denmat_dynm_development_gb300.dmd import LindbladGPU
    return LindbladGPU(nk=s.nk, nb_dm=s.nb_dm, bstart=s.bstart, bend=s.bend, e_dm=s.e_dm, k1st=s.k1st, k2nd=s.k2nd,
                       P1=kw.pop("P1", s.P1), P2=kw.pop("P2", s.P2), prefac_eph=s.prefac_eph, Hcoh=s.Hcoh,
                       picture=s.picture_schrodinger, expt=s.expt, precision="f64", sparse=True, **kw)


@pytest.mark.parametrize("case", SPARSE_CASES + ["nb4_eimp_B", "nb2_window"])
def test_sparse_rhs_and_rk4_vs_golden(case, oracle, built):
    d = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(d, "golden.npz")))
    s = oracle.load(d)
    with make_sparse(s) as gpu:
        for i, t in enumerate(g["rhs_t"]):
            y = g["rhs_y"][i]
            e1 = rel(gpu.func(t, y), g["rhs_dydt"][i])
            e2 = rel(gpu.evolve_driver(t, y), g["rhs_eph"][i])
            print("%s t=%g: RHS rel err %.3g, scattering term %.3g" % (case, t, e1, e2))
            assert e1 < 1e-12 and e2 < 1e-12
        gpu.set_state(s.t0, oracle.y_of(s.dm0))
        gpu.rk4(1.0 * oracle.fs, 40)
        _, y = gpu.get_state()
        assert rel(y, g["rk4_y"]) < 1e-10


@pytest.mark.parametrize("case", SPARSE_CASES)
def test_sparse_rkf45_matches_reference_loop(case, oracle, built):
    """DMD's evolve_gsl (RKF45, y_new control) with the sparse contraction: the S_z record and the
    RHS-call counts of the reference's own sparse run."""
    d = os.path.join(GOLDEN, case)
    g = dict(np.load(os.path.join(d, "golden.npz")))
    s = oracle.load(d)
    with make_sparse(s) as gpu:
        gpu.set_state(s.t0, oracle.y_of(s.dm0))
        gpu.set_observable(0, s.smat[:, 2, :], s.f_dm, s.ob_prefac)
        hs = s.ode["hstart"]
        ti = tcur = s.t0
        sz, nf = [], []
        while tcur < s.tend:
            ti += s.tstep
            hs, n = gpu.rkf45_apply(ti, hs, s.ode["hmin"], s.ode["hmax"], s.ode["epsabs"], 0.0)
            tcur, _ = gpu.get_state()
            sz.append(gpu.measure(0, s.nv_dm)[0])
            nf.append(n)
        _, y = gpu.get_state()
    assert rel(y, g["gsl_y"]) < 1e-10
    assert rel(np.array(sz), g["gsl_sz"][1:, 1]) < 1e-10
    np.testing.assert_array_equal(np.array(nf), g["gsl_ncalls"])


def test_sparse_with_structural_zeros_and_additive_operators(oracle, built):
    """Operators with 80 % structural zeros plus additive (e-imp) operators with their own zeros: the
    sparse form folds P + scale P_add in FP64 before it filters the elements, as the dense forms
    fold; against the oracle's dense RHS of the folded operators."""
    s = oracle.load(os.path.join(GOLDEN, "nb4_eimp_B"))
    rng = np.random.default_rng(4)
    nb4 = (s.bend - s.bstart) ** 4
    P1 = s.P1.reshape(-1, nb4).copy()
    P2 = s.P2.reshape(-1, nb4).copy()
    m = rng.random(P1.shape) < 0.8
    P1[m] = 0
    P2[m] = 0
    A1 = np.where(rng.random(P1.shape) < 0.9, 0, 1e-2 * (rng.standard_normal(P1.shape) + 1j * rng.standard_normal(P1.shape)))
    A2 = np.conj(A1[:, ::-1])
    scale = 0.37
    s.P1 = np.ascontiguousarray((P1 + scale * A1).reshape(-1))
    s.P2 = np.ascontiguousarray((P2 + scale * A2).reshape(-1))
    t = 11.0 * oracle.fs
    y = oracle.y_of(s.dm0)
    with make_sparse(s, P1=P1.reshape(-1), P2=P2.reshape(-1), P1_add=A1.reshape(-1), P2_add=A2.reshape(-1),
                     add_scale=scale) as gpu:
        e = rel(gpu.func(t, y), oracle.rhs(s, t, y))
        nbytes = gpu.pair_bytes
    print("80 %% zeros + additive operators: RHS rel err %.3g, %d stored bytes vs %d dense"
          % (e, nbytes, s.npair * 2 * nb4 * 16))
    assert e < 1e-12
    assert nbytes < s.npair * 2 * nb4 * 16


def test_sparse_operator_files(oracle, built, tmp_path, monkeypatch):
    """DMD's sparse operator files (alg.Pin_is_sparse) read straight into the sparse form, in chunks
    of 5 pairs, equal the same operators given as dense arrays to the dense FP64 form."""
    from denmat_dynm_development_gb300.dmd import LindbladGPU
    s = oracle.load(os.path.join(GOLDEN, "nb4_sparse"))
    rng = np.random.default_rng(8)
    nb4 = (s.bend - s.bstart) ** 4
    monkeypatch.setenv("DMD_FILL_CHUNK", "5")
    sp = [write_sparse(str(tmp_path / n), P, nb4, rng) for n, P in (("sP1", s.P1), ("sP2", s.P2))]
    kw = dict(nk=s.nk, nb_dm=s.nb_dm, bstart=s.bstart, bend=s.bend, e_dm=s.e_dm, k1st=s.k1st, k2nd=s.k2nd,
              prefac_eph=s.prefac_eph, Hcoh=s.Hcoh, picture=s.picture_schrodinger, expt=s.expt, precision="f64")
    y = oracle.y_of(s.dm0)
    t = 31.0 * oracle.fs
    with LindbladGPU(P1=s.P1, P2=s.P2, **kw) as gd:
        rd = gd.func(t, y)
    with LindbladGPU(P1=None, P2=None, P_sparse=sp, sparse=True, **kw) as gs:
        r = gs.func(t, y)
    assert rel(r, rd) < 1e-13
    assert rel(r, oracle.rhs(s, t, y)) < 1e-12


@pytest.mark.parametrize("nb_dm,bstart,bend,npair,picture", [(3, 0, 3, 150, 0), (1, 0, 1, 80, 1), (3, 1, 2, 50, 1),
                                                             (2, 0, 2, 0, 0), (4, 0, 4, 90, 0)])
def test_sparse_windows_and_empty_pairs(nb_dm, bstart, bend, npair, picture, oracle, built):
    """nb = 1, 3 windows (one inside the density matrix), an empty pair list and nb = 4, with half the
    elements of the random operators zeroed: RHS and 5 RK4 steps against the oracle."""
    s = _random_system(oracle, 23, nb_dm, bstart, bend, npair, seed=nb_dm * 10 + npair + 3, picture=picture)
    rng = np.random.default_rng(npair + 1)
    z = rng.random(s.P1.shape) < 0.5
    s.P1 = np.where(z, 0, s.P1)
    s.P2 = np.where(z, 0, s.P2)
    y = oracle.y_of(s.dm0)
    t = 5.0 * oracle.fs
    with make_sparse(s) as gpu:
        e = rel(gpu.func(t, y), oracle.rhs(s, t, y))
        gpu.set_state(0.0, y)
        gpu.rk4(1.0 * oracle.fs, 5)
        _, yg = gpu.get_state()
    yo, _ = oracle.rk4(s, 0.0, 1.0 * oracle.fs, 5, y)
    assert e < 1e-12
    assert rel(yg - y, yo - y) < 1e-11


def test_sparse_non_hermitian_state(oracle, built):
    """The GSL callback may pass any y: the sparse form contracts the complex coordinates directly."""
    s = oracle.load(os.path.join(GOLDEN, "nb4_sparse"))
    rng = np.random.default_rng(3)
    dm = s.dm0 + 1e-3 * (rng.standard_normal(s.dm0.shape) + 1j * rng.standard_normal(s.dm0.shape))
    y = oracle.y_of(dm)
    t = 13.0 * oracle.fs
    with make_sparse(s) as gpu:
        assert rel(gpu.func(t, y), oracle.rhs(s, t, y)) < 1e-12
