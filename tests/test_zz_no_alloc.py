"""The allocation-free entry point dmd_evolve_driver_noalloc against the allocating one.

dmd_evolve_driver_noalloc serves callers that cannot allocate device memory (graph captures,
frameworks whose pools own the device, plug-ins given device pointers only); its scratch is a static
device array. Here the test plays such a caller: it owns the device buffers (made with torch), calls
the entry point twice in a row through the C ABI on different states and times, and compares each
result with dmd_evolve_driver (host-buffer entry point) at the FP64 RHS tolerance, 1e-12 normwise,
and, on the golden states, with the reference's own scattering term (the fixture's rhs_eph). This
file is collected last so that a failure here leaves every other test already run; it must also pass
on its own in a fresh process. The size check runs without a GPU.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["nb2_eimp_B", "nb4_eimp_B", "nb2_window"])
def test_noalloc_matches_allocating_entry_point(case, oracle):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as G
    G.build()
    from denmat_dynm_development_gb300.dmd import LindbladGPU, _lib
    L = _lib()
    s = oracle.load(os.path.join(GOLDEN, case))
    dev = torch.device("cuda:0")
    # caller-owned device buffers in DMD's own layouts
    k1 = torch.from_numpy(s.k1st.view(np.int64).copy()).to(dev)
    k2 = torch.from_numpy(s.k2nd.view(np.int64).copy()).to(dev)
    P1 = torch.from_numpy(s.P1.view(np.float64).copy()).to(dev)
    P2 = torch.from_numpy(s.P2.view(np.float64).copy()).to(dev)
    e = torch.from_numpy(s.e_dm.copy()).to(dev)
    ny = 2 * s.nk * s.nb_dm * s.nb_dm
    dm = torch.zeros(ny, dtype=torch.float64, device=dev)
    out = torch.zeros(ny, dtype=torch.float64, device=dev)
    rng = np.random.default_rng(7)
    ref = LindbladGPU(nk=s.nk, nb_dm=s.nb_dm, bstart=s.bstart, bend=s.bend, e_dm=s.e_dm, k1st=s.k1st, k2nd=s.k2nd,
                      P1=s.P1, P2=s.P2, prefac_eph=s.prefac_eph, expt=s.expt, precision="f64")
    try:
        for t in (0.0, 37.0 * oracle.fs):  # two calls in a row; the second reuses the shared scratch
            d = s.dm0 + 1e-3 * (rng.standard_normal(s.dm0.shape) + 1j * rng.standard_normal(s.dm0.shape))
            d = d.reshape(s.nk, s.nb_dm, s.nb_dm)
            d = 0.5 * (d + np.conj(np.swapaxes(d, 1, 2)))
            y = np.ascontiguousarray(d.reshape(s.nk, -1)).view(np.float64).reshape(-1)
            dm.copy_(torch.from_numpy(y))
            out.fill_(np.nan)
            stream = torch.cuda.current_stream(dev).cuda_stream
            st = L.dmd_evolve_driver_noalloc(s.nk, s.nb_dm, s.bstart, s.bend, s.npair, k1.data_ptr(), k2.data_ptr(),
                                             P1.data_ptr(), P2.data_ptr(), e.data_ptr(), s.prefac_eph, s.expt, t,
                                             dm.data_ptr(), out.data_ptr(), C.c_void_p(stream))
            assert st == 0
            torch.cuda.synchronize(dev)
            got = out.cpu().numpy()
            want = ref.evolve_driver(t, y)
            assert rel(got, want) < 1e-12
        # the golden states against the reference's own evolve_driver output
        g = dict(np.load(os.path.join(GOLDEN, case, "golden.npz")))
        for i, t in enumerate(g["rhs_t"]):
            dm.copy_(torch.from_numpy(np.ascontiguousarray(g["rhs_y"][i])))
            out.fill_(np.nan)
            stream = torch.cuda.current_stream(dev).cuda_stream
            st = L.dmd_evolve_driver_noalloc(s.nk, s.nb_dm, s.bstart, s.bend, s.npair, k1.data_ptr(), k2.data_ptr(),
                                             P1.data_ptr(), P2.data_ptr(), e.data_ptr(), s.prefac_eph, s.expt,
                                             float(t), dm.data_ptr(), out.data_ptr(), C.c_void_p(stream))
            assert st == 0
            torch.cuda.synchronize(dev)
            assert rel(out.cpu().numpy(), g["rhs_eph"][i]) < 1e-12
    finally:
        ref.close()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    """Runs in the CPU suite too: the size check comes before any CUDA call."""
    import __graft_entry__ as G
    G.build()
    from denmat_dynm_development_gb300.dmd import _lib
    L = _lib()
    # nk * nb^2 above 262144 is refused before any device work (null pointers are never touched)
    dummy = C.c_void_p(16)
    st = L.dmd_evolve_driver_noalloc(70000, 2, 0, 2, 0, None, None, None, None, dummy, 1.0, 1, 0.0, dummy, dummy, None)
    assert st == 1
