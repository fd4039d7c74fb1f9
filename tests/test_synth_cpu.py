"""The synthetic generator's streamed operator sets (CPU): what the adjoint of the 4.19M-pair
MoS2-like system uses in place of holding every phonon mode's operators at once."""
import numpy as np


def test_streamed_mode_sets_equal_the_in_memory_ones():
    """ldbd_synth.ModeSets (worker processes, chunk by chunk, shared memory) gives the operator sets
    of mode_operators, their theta-weighted sum and the contractions Re sum conj(G) P^(m)."""
    from denmat_dynm_development_gb300 import ldbd_synth as S
    cfg = S.SynthConfig(nk=60, nb=4, seed=9, de_pair_mev=60.0, eimp_sigma_mev=5.0)
    st, P1m, P2m, Q1, Q2 = S.mode_operators(cfg)
    A1 = np.concatenate([P1m, Q1[None]])
    A2 = np.concatenate([P2m, Q2[None]])
    ms = S.ModeSets(cfg, procs=2)
    assert ms.nparams == A1.shape[0] and ms.st.npair == st.npair
    for m in (0, ms.nparams - 1):
        p = ms.mode(m)
        try:
            np.testing.assert_array_equal(p.a[0], A1[m])
            np.testing.assert_array_equal(p.a[1], A2[m])
        finally:
            p.close()
    th = np.linspace(0.5, 1.5, ms.nparams)
    p = ms.scaled(th)
    try:
        np.testing.assert_allclose(p.a[0], np.tensordot(th, A1, 1), rtol=0, atol=1e-15 * np.abs(A1).max())
        rng = np.random.default_rng(1)
        G = S.SharedPair(st.npair, cfg.nb ** 4)
        try:
            G.a[...] = rng.standard_normal(G.a.shape) + 1j * rng.standard_normal(G.a.shape)
            got = ms.contract(G)
            want = np.array([np.vdot(G.a[0], A1[m]).real + np.vdot(G.a[1], A2[m]).real for m in range(ms.nparams)])
            np.testing.assert_allclose(got, want, rtol=1e-12)
        finally:
            G.close()
    finally:
        p.close()
