"""Generates the committed fixtures under tests/golden/ from the reference.

restart_30x30x60.npz: the reference's own state fixture, bin/restart.nc
(30x30x60, FP64, iteration 105000), read with scipy's NetCDF reader.  GPU
tests start parity runs from it, since the reference tree is not present on
the machine that runs them.

reference_inputs.json: the text of the reference's three parameter files
(bin/INPUT, bin/originalINPUT, bin/test1/INPUT), which the CPU tests parse
through the library's INPUT reader.

Usage (from the repository root, with the reference's VarElecCond directory
given as the argument or in VEC_REFERENCE_DIR):
    python tests/golden/make_fixtures.py <reference>/VarElecCond
"""
import json
import os
import sys

import numpy as np
from scipy.io import netcdf_file

FIELDS = ("R", "T", "U", "V", "W", "Bx", "By", "Bz")
ATTRS = ("gamma", "sigma", "theta", "ck", "cm", "f", "tayl", "psi", "zeta", "xmax", "ymax")
INPUTS = ("INPUT", "originalINPUT", "test1/INPUT")


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
    texts = {}
    for sub in INPUTS:
        with open(os.path.join(refdir, "bin", sub)) as f:
            texts[sub] = f.read()
    with open(os.path.join(here, "reference_inputs.json"), "w") as f:
        json.dump(texts, f, indent=1)


if __name__ == "__main__":
    d = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VEC_REFERENCE_DIR")
    if not d:
        sys.exit("usage: make_fixtures.py <reference VarElecCond directory> (or set VEC_REFERENCE_DIR)")
    main(d)
