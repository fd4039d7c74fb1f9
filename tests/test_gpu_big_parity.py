"""Parity at the benchmarked sizes (GPU; the oracle side runs split over all host cores).

One RHS of the 9.7M-pair GaAs-like benchmark workload and a 200-step RK4 trajectory of the Si-like
nk = 500 system, GPU against the oracle, in the plain FP64 form and the FP32-pair form. The work runs
in a child interpreter (tests/big_parity_child.py) so that the oracle's forked worker processes start
before any CUDA call. Tolerances: RHS 1e-12 (f64) / 1e-11 (f64x), trajectory and S_z 1e-10 -- the
bounds the fixtures are held to.
"""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def big():
    import __graft_entry__ as G
    G.build()
    p = subprocess.run([sys.executable, os.path.join(HERE, "big_parity_child.py")], capture_output=True, text=True,
                       timeout=900)
    sys.stdout.write(p.stdout[-2000:])
    sys.stderr.write(p.stderr[-4000:])
    assert p.returncode == 0, p.stderr[-2000:]
    line = [x for x in p.stdout.splitlines() if x.startswith("RESULT ")][-1]
    r = json.loads(line[len("RESULT "):])
    print(r)
    return r


@pytest.mark.parametrize("prec,tol", [("f64", 1e-12), ("f64x", 1e-11)])
def test_rhs_at_benchmark_size(big, prec, tol):
    assert big["npair_gaas_nk20k"] > 9_000_000
    assert big["rhs_gaas_nk20k_" + prec] < tol


@pytest.mark.parametrize("prec", ["f64", "f64x"])
def test_rk4_200_steps_si_nk500(big, prec):
    assert big["rk4_si_nk500_200_" + prec] < 1e-10
    assert big["sz_si_nk500_200_" + prec] < 1e-10


def test_host_rk4_driver_at_benchmark_size(big):
    """dmdh_rk4_func (host stage loops split over threads at this size) equals the device RK4 loop"""
    assert big["host_rk4_vs_device_gaas_nk20k"] < 1e-13
