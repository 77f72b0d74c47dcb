"""Generates the committed fixtures under tests/golden/ from the reference.

restart_30x30x60.npz: the reference's own state fixture, bin/restart.nc
(30x30x60, FP64, iteration 105000), read with scipy's NetCDF reader.  GPU
tests start parity runs from it, since the reference tree is not present on
the machine that runs them.

Usage (from the repository root, with the reference mounted):
    python tests/golden/make_fixtures.py /root/reference/VarElecCond
"""
import os
import sys

import numpy as np
from scipy.io import netcdf_file

FIELDS = ("R", "T", "U", "V", "W", "Bx", "By", "Bz")
ATTRS = ("gamma", "sigma", "theta", "ck", "cm", "f", "tayl", "psi", "zeta", "xmax", "ymax")


def main(refdir):
    here = os.path.dirname(os.path.abspath(__file__))
    with netcdf_file(os.path.join(refdir, "bin", "restart.nc"), "r", mmap=False) as f:
        out = {n: np.asarray(f.variables[n][:], dtype=np.float64) for n in FIELDS}
        out["time"] = np.float64(f.variables["time"][0])
        out["iteration"] = np.int64(f.variables["iteration"][0])
        out["timestep"] = np.float64(f.variables["timestep"][0])
        for a in ATTRS:
            out[a] = np.float64(getattr(f, a))
    np.savez_compressed(os.path.join(here, "restart_30x30x60.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/VarElecCond")
