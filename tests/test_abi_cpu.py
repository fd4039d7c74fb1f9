"""CPU-only checks of the native boundary: the libraries build, load, and export every symbol the
public headers declare; argument validation answers without touching a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dmd_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def gpu_lib():
    from denmat_dynm_development_gb300 import build as B
    path = B.build_gpu()
    return C.CDLL(path)


def test_gpu_lib_exports_header(gpu_lib):
    names = declared("dmd_gpu.h")
    assert "dmd_create" in names and "dmd_func" in names
    missing = [n for n in names if not hasattr(gpu_lib, n)]
    assert not missing, missing


def test_python_binding_lists_all_exports():
    from denmat_dynm_development_gb300 import dmd
    assert sorted(dmd.EXPORTS) == declared("dmd_gpu.h")


def test_strerror_and_null_arguments(gpu_lib):
    gpu_lib.dmd_strerror.restype = C.c_char_p
    assert gpu_lib.dmd_strerror(0) == b"ok"
    assert gpu_lib.dmd_strerror(1) == b"invalid argument"
    # a null descriptor is rejected before any device call
    h = C.c_void_p()
    assert gpu_lib.dmd_create(None, C.byref(h)) == 1
    assert gpu_lib.dmd_destroy(None) == 1


def test_create_from_files_rejects_wrong_sizes(tmp_path):
    """a file whose size is not nkpair * nb^4 * 16 bytes gives DMD_E_FILE before any device work"""
    import ctypes as C
    from denmat_dynm_development_gb300 import dmd
    L = dmd._lib()
    good = tmp_path / "P1.bin"
    bad = tmp_path / "P2.bin"
    np.zeros(5 * 16, np.complex128).tofile(str(good))
    np.zeros(5 * 16 - 1, np.complex128).tofile(str(bad))
    d = dmd._Desc(nk=10, nb_dm=2, bstart=0, bend=2, nkpair=5)
    h = C.c_void_p()
    st = L.dmd_create_from_files(C.byref(d), str(good).encode(), str(bad).encode(), None, None, C.byref(h))
    assert st == 3  # DMD_E_FILE
    st = L.dmd_create_from_files(C.byref(d), str(good).encode(), str(tmp_path / "missing").encode(), None, None,
                                 C.byref(h))
    assert st == 3


def test_create_from_sparse_files_checks_the_counts_file(tmp_path):
    """the per-pair count file must hold one int32 per k-pair (DMD_E_FILE before any device work)"""
    import ctypes as C
    from denmat_dynm_development_gb300 import dmd
    L = dmd._lib()
    for m in ("sP1", "sP2"):
        np.zeros(4, np.int32).tofile(str(tmp_path / (m + "_ns.bin")))  # 4 counts for 5 pairs
        for sfx in ("_s.bin", "_i.bin", "_j.bin"):
            open(str(tmp_path / (m + sfx)), "wb").close()
    d = dmd._Desc(nk=10, nb_dm=2, bstart=0, bend=2, nkpair=5)
    h = C.c_void_p()
    st = L.dmd_create_from_sparse_files(C.byref(d), str(tmp_path / "sP1").encode(), str(tmp_path / "sP2").encode(),
                                        None, None, C.byref(h))
    assert st == 3  # DMD_E_FILE


def test_sparse_flag_is_validated_before_any_device_call():
    """DMD_FLAG_SPARSE is the FP64 form of one state without the linearized, adjoint or e-e options:
    other combinations give DMD_E_ARG before the device is queried"""
    import ctypes as C
    from denmat_dynm_development_gb300 import dmd
    L = dmd._lib()
    e = np.zeros((4, 2))
    k = np.zeros(1, np.uint64)
    P = np.zeros(16, np.complex128)
    h = C.c_void_p()
    for prec, flags, nrhs in ((dmd.PREC["f64x"], dmd.FLAG_SPARSE, 1), (dmd.PREC["f64"], dmd.FLAG_SPARSE | dmd.FLAG_ADJOINT, 1),
                              (dmd.PREC["f64"], dmd.FLAG_SPARSE | dmd.FLAG_EE, 1), (dmd.PREC["f32"], dmd.FLAG_SPARSE, 4)):
        d = dmd._Desc(nk=4, nb_dm=2, bstart=0, bend=2, nkpair=1, e_dm=e.ctypes.data, k1st=k.ctypes.data,
                      k2nd=k.ctypes.data, P1=P.ctypes.data, P2=P.ctypes.data, precision=prec, flags=flags, nrhs=nrhs)
        assert L.dmd_create(C.byref(d), C.byref(h)) == 1


def test_binding_refuses_to_run_without_its_library(monkeypatch):
    """the Python binding has no host fallback: a missing libdmdgpu.so is an error at first use"""
    from denmat_dynm_development_gb300 import dmd
    monkeypatch.setattr(dmd, "_L", None)
    monkeypatch.setattr(dmd, "GPU_LIB", os.path.join(ROOT, "no_such_dir", "libdmdgpu.so"))
    with pytest.raises(RuntimeError, match="not built"):
        dmd.LindbladGPU(nk=1, nb_dm=1, bstart=0, bend=1, e_dm=np.zeros(1), k1st=np.zeros(1, np.uint64),
                        k2nd=np.zeros(1, np.uint64), P1=np.zeros(1, np.complex128), P2=np.zeros(1, np.complex128),
                        prefac_eph=1.0)


@pytest.mark.skipif(os.path.exists("/dev/nvidia0"), reason="a GPU is present: the handle is created there")
def test_create_without_a_device_is_an_error_not_a_host_path():
    """with no CUDA device a valid descriptor gives DMD_E_NODEV (or DMD_E_CUDA): nothing is computed
    on the host instead"""
    from denmat_dynm_development_gb300 import dmd
    nk, nb = 2, 2
    e = np.array([[0.0, 0.01], [0.002, 0.012]])
    with pytest.raises(dmd.DMDError) as ei:
        dmd.LindbladGPU(nk=nk, nb_dm=nb, bstart=0, bend=nb, e_dm=e, k1st=np.array([0], np.uint64),
                        k2nd=np.array([1], np.uint64), P1=np.zeros(nb ** 4, np.complex128),
                        P2=np.zeros(nb ** 4, np.complex128), prefac_eph=1.0)
    assert ei.value.status in (4, 8)


C_CALLER = r"""
#include <stdio.h>
#include <string.h>
#include "dmd_gpu.h"
#include "dmd_host.h"

int main(void) {
  dmd_handle* h = 0;
  dmdh_system* s = 0;
  double e[3] = {-0.01, 0.0, 0.01}, f[3];
  if (strcmp(dmd_strerror(DMD_OK), "ok") != 0) return 1;
  if (dmd_create(0, &h) != DMD_E_ARG) return 2;              /* null descriptor */
  if (dmdh_load("/nonexistent/ldbd/dir", &s) == 0) return 3; /* missing inputs */
  if (dmdh_error() == 0 || dmdh_error()[0] == 0) return 4;
  if (dmdh_fermi(1e-3, 0.0, e, f, 3) != 0) return 5;         /* host arithmetic, no device */
  printf("%.17g %.17g %.17g\n", f[0], f[1], f[2]);
  return 0;
}
"""


def test_plain_c_caller_links_and_calls_the_abi(tmp_path):
    """The public headers are plain C (C99, no C++ types): a C program includes both, links
    libdmdgpu.so and libdmdhost.so, and calls entry points that need no device"""
    import shutil
    import subprocess
    from denmat_dynm_development_gb300 import build as B
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    B.build_gpu()
    B.build_host()
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(B.GPU_LIB)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-o", str(exe), "-L", libdir, "-ldmdhost", "-ldmdgpu", "-Wl,-rpath," + libdir],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, (out.returncode, out.stderr)
    f = np.array([float(x) for x in out.stdout.split()])
    from denmat_dynm_development_gb300 import host as H
    np.testing.assert_array_equal(f, H.fermi(1e-3, 0.0, np.array([-0.01, 0.0, 0.01])))
