"""Golden vectors for the T1 fit, taken from the reference's shipped GaAs example run.

The example directory (eph-ei, n2e16_ni2e16) holds the S_z(t) trajectory DMD wrote
(sz_elec_tot.out) and what the reference's fit.py made of it (sfit.out: t, S, fitted S over the
first 3.2 ps; tau_t.dat: two-point log-fit lifetimes). This script copies the numeric columns into
t1_gaas_example.npz; it reads the reference tree and runs only where that tree exists.

    python tests/golden/make_t1_golden.py [REFERENCE_ROOT]

(REFERENCE_ROOT defaults to $DMD_REFERENCE_ROOT, itself defaulting to /root/reference)
"""
import os
import sys

import numpy as np

EXAMPLE = "Examples/RealTime_Example_GaAs_20230105/ld-dmd/t300/mult8_gauss0.005/dBz/eph-ei/n2e16_ni2e16"


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DMD_REFERENCE_ROOT", "/root/reference")
    d = os.path.join(ref, EXAMPLE)
    sz = np.loadtxt(os.path.join(d, "sz_elec_tot.out"))
    sfit = np.loadtxt(os.path.join(d, "sfit.out"))
    tau_t = np.loadtxt(os.path.join(d, "tau_t.dat"))
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "t1_gaas_example.npz")
    np.savez_compressed(out, sz=sz, sfit=sfit, tau_t=tau_t)
    print("wrote", out, sz.shape, sfit.shape, tau_t.shape)


if __name__ == "__main__":
    main()
