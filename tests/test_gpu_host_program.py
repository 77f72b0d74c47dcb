"""The C host program p3d_gpu (src/main.F90 on the GPU library) against the
oracle: its printed diagnostics blocks (src/main.F90:552-647) line by line.

The reference's CPU-runnable case (64^2 x 65, Ra 1e5, Q 100, eta contrast
5, fixed-flux bottom, +-1e-3 noise) is written as a reference INPUT file
(src/initial.F90:94-201), run for 200 steps with diagnostics every 50, and
every value of every printed block -- the time, ubar, vbar, the div B
extrema, the Alfven, Mach and rms extrema, the field extrema, the magnetic
and kinetic energies and the Nusselt number -- is compared with the
oracle's diagnostics at the same steps.  The program prints 17 significant
digits, as Fortran list-directed output does.

Tolerance: 1e-9 relative plus 1e-12 absolute (the smallest Mach number is
the slowest point's speed, ~1e-7, whose last digits are rounding), and
1e-11 absolute for the values that are rounding noise on both sides (ubar
and vbar after GlobalAverages removed the mean momentum, div B).
"""
import os
import re
import subprocess

import pytest

from oracle import oracle as O
from fug30v0kxc_gb300.solver import read_input

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROG = os.path.join(ROOT, "fug30v0kxc_gb300", "_lib", "p3d_gpu")

INPUT = """data file for the compressible magnetoconvection program

2\t     INPUT FLAG (1 for CK/F, 2 for Ra/Q)

VALUE        VARIABLE
1.4      GAMMA
1.00          SIGMA
9.0         THETA
100000.0      CK (if FLAG=1) or Ra (if FLAG=2)
1.0          CM
100.0          F (if FLAG=1) or Q (if FLAG=2)
0.0      TAYL (mid layer)
1.570796327         PSI
0.2          ZETA
4.0          XMAX
4.0          YMAX
0.3          SF
0            NFRAME
200       TOTAL
50          NDU06
1000000        NDU16
10            NDURESTART
64\t     NX
64\t     NY
65\t     NZ
"""
NAMES = {"magenergy": "menergy", "kinenergy": "kenergy", "Nusselt": "nusselt"}


def _blocks(out):
    """(nit, ttime, {name: value}) per printed diagnostics block."""
    res = []
    for blk in out.split(" NIT= ")[1:]:
        m = re.match(r"\s*(\d+)\s+TTIME\s+(\S+)", blk)
        vals = {NAMES.get(k, k): float(v) for k, v in re.findall(r"(\w+)=\s+(\S+)", blk)}
        res.append((int(m.group(1)), float(m.group(2)), vals))
    return res


def test_printed_diagnostics_match_oracle(tmp_path):
    (tmp_path / "INPUT").write_text(INPUT)
    r = subprocess.run([PROG, "--constflux", "--eta-contrast", "5", "--noise", "1e-3"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    blocks = _blocks(r.stdout)
    assert [b[0] for b in blocks] == [50, 100, 150, 200]

    p = read_input(str(tmp_path / "INPUT"))
    p.constflux, p.eta_contrast, p.noise_amp = 1, 5.0, 1e-3
    o = O.Oracle(p)
    o.start()
    for nit, ttime, vals in blocks:
        assert o.step(50) == 0
        ref = o.last_diag()
        assert abs(ttime - o.scalars().ttime) <= 1e-12 * abs(o.scalars().ttime), nit
        assert len(vals) == 29, sorted(vals)
        for k, v in vals.items():
            b = ref[k]
            floor = 1e-11 if k in ("ubar", "vbar", "divbmin", "divbmax") else 1e-12
            assert abs(v - b) <= 1e-9 * abs(b) + floor, (nit, k, v, b)
    o.close()
