"""The reference's multi-rank decomposition of the RHS, run as two gloo ranks on the CPU.

DMD splits the stored k-pairs into contiguous slices per MPI rank (mymp::distribute_var,
comm/mymp.cpp:8-36), every rank accumulates partial Pdm / dm1P over its slice, an allreduce sums
them (evolve_eph.cpp:137) and every rank finishes all k. A multi-GPU form of this path shards the
same way with one exchange step per RHS. Here two torch.distributed gloo ranks play the MPI ranks:
each computes its slice with the oracle, all_reduce sums the partials, and the finished RHS must
equal the single-process rank-sliced RHS bit for bit and the one-rank RHS to rounding.
"""
import os
import socket

import numpy as np
import pytest

from conftest import GOLDEN, ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, case, t, out_dir):
    import ctypes as C
    import sys
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    from oracle import oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        s = O.load(os.path.join(GOLDEN, case))
        g = dict(np.load(os.path.join(GOLDEN, case, "golden.npz")))
        y = np.ascontiguousarray(g["rhs_y"][1])
        L = O.lib()
        nb = s.bend - s.bstart
        e_w = np.zeros((s.nk, nb))
        dm_w = np.zeros((s.nk, nb * nb), np.complex128)
        dm1_w = np.zeros_like(dm_w)
        cs = s.cstruct()
        L.orc_window_in(C.addressof(cs), y.ctypes.data, e_w.ctypes.data, dm_w.ctypes.data, dm1_w.ctypes.data)
        n = s.npair
        p0, p1 = (n * rank) // world, (n * (rank + 1)) // world
        part = np.zeros((2, s.nk, nb * nb), np.complex128)
        L.orc_pairs_partial(C.addressof(cs), e_w.ctypes.data, t, dm_w.ctypes.data, dm1_w.ctypes.data, p0, p1,
                            part[0].ctypes.data, part[1].ctypes.data)
        buf = torch.from_numpy(part.view(np.float64).copy())
        dist.all_reduce(buf, op=dist.ReduceOp.SUM)
        tot = buf.numpy().view(np.complex128)
        Pdm, dm1P = np.ascontiguousarray(tot[0]), np.ascontiguousarray(tot[1])
        out = np.zeros_like(y)
        L.orc_rhs_from_partials(C.addressof(cs), t, y.ctypes.data, e_w.ctypes.data, dm_w.ctypes.data,
                                dm1_w.ctypes.data, Pdm.ctypes.data, dm1P.ctypes.data, out.ctypes.data)
        np.save(os.path.join(out_dir, "rank%d.npy" % rank), out)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("case", ["nb2_eimp_B", "nb4_eimp_B"])
def test_two_gloo_ranks_match_rank_sliced_rhs(case, oracle, tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    if not torch.distributed.is_available() or not torch.distributed.is_gloo_available():
        pytest.skip("gloo backend unavailable")
    g = dict(np.load(os.path.join(GOLDEN, case, "golden.npz")))
    t = float(g["rhs_t"][1])
    mp.spawn(_rank_main, args=(2, _free_port(), case, t, str(tmp_path)), nprocs=2, join=True)
    r0 = np.load(str(tmp_path / "rank0.npy"))
    r1 = np.load(str(tmp_path / "rank1.npy"))
    np.testing.assert_array_equal(r0, r1)          # every rank holds the full result
    # the same two slices summed in one process (p0 + p1) is the same arithmetic
    import ctypes as C
    s = oracle.load(os.path.join(GOLDEN, case))
    L = oracle.lib()
    cs = s.cstruct()
    y = np.ascontiguousarray(g["rhs_y"][1])
    nb = s.bend - s.bstart
    e_w = np.zeros((s.nk, nb))
    dm_w = np.zeros((s.nk, nb * nb), np.complex128)
    dm1_w = np.zeros_like(dm_w)
    L.orc_window_in(C.addressof(cs), y.ctypes.data, e_w.ctypes.data, dm_w.ctypes.data, dm1_w.ctypes.data)
    n = s.npair
    parts = []
    for p0, p1 in ((0, n // 2), (n // 2, n)):
        Pdm = np.zeros_like(dm_w)
        dm1P = np.zeros_like(dm_w)
        L.orc_pairs_partial(C.addressof(cs), e_w.ctypes.data, t, dm_w.ctypes.data, dm1_w.ctypes.data, p0, p1,
                            Pdm.ctypes.data, dm1P.ctypes.data)
        parts.append((Pdm, dm1P))
    Pdm = parts[0][0] + parts[1][0]
    dm1P = parts[0][1] + parts[1][1]
    want = np.zeros_like(y)
    L.orc_rhs_from_partials(C.addressof(cs), t, y.ctypes.data, e_w.ctypes.data, dm_w.ctypes.data,
                            dm1_w.ctypes.data, Pdm.ctypes.data, dm1P.ctypes.data, want.ctypes.data)
    np.testing.assert_array_equal(r0, want)
    ref = g["rhs_dydt"][1]
    assert np.abs(r0 - ref).max() <= 1e-13 * np.abs(ref).max()
