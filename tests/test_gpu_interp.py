"""The interpolate program (interpolate/main.F90) as the C host interp_gpu:
restart.nc (nx, ny, nz) -> output.nc (2 nx, 2 ny, nz), every field the
spectral expand of interpolate/fft.F90:834-927.  Checked against the numpy
restatement of expand to 1e-12 of each field's scale; output.nc has 64-bit
offsets and double fields as the reference writes it."""
import os
import subprocess

import numpy as np
import pytest

from oracle import closure_oracle as CO
from fug30v0kxc_gb300.build import INTERP
from fug30v0kxc_gb300.solver import SNAP_ATTRS, SNAP_FIELDS, nc_read, nc_write
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu


def test_interp_program_expands_a_snapshot(tmp_path):
    nx, ny, nz = 32, 16, 7
    rng = np.random.default_rng(9)
    snap = {}
    for n in SNAP_FIELDS:
        snap[n] = rng.standard_normal((nz, ny, nx))
    snap["R"] = 2.0 + 0.1 * snap["R"]
    snap["T"] = 3.0 + 0.1 * snap["T"]
    snap.update(time=2.5, iteration=1234, timestep=1e-4, version=3, history="interp test")
    attrs = dict(gamma=1.4, sigma=1.0, theta=9.0, ck=0.05, cm=1.0, f=0.1, tayl=0.0, psi=1.5707963, zeta=0.2,
                 xmax=4.0, ymax=4.0)
    snap.update(attrs)
    nc_write(tmp_path / "restart.nc", snap, 8)
    r = subprocess.run([INTERP], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "TTIME" in r.stdout and "bzmax=" in r.stdout
    assert open(tmp_path / "output.nc", "rb").read(4) == b"CDF\x02"
    out = nc_read(tmp_path / "output.nc")
    assert out["iteration"] == 1234 and out["time"] == 2.5
    for n in SNAP_FIELDS:
        assert out[n].shape == (nz, 2 * ny, 2 * nx)
        assert rel_err(out[n], CO.expand(snap[n], 2)) < 1e-12, n
    for a in SNAP_ATTRS:
        assert out[a] == snap[a]
