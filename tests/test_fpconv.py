"""The integer-pipe float <-> double conversions (csrc/fpconv.cuh) compiled
for the host and checked bit for bit against the C casts."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "fug30v0kxc_gb300", "csrc")


def test_fpconv_matches_casts(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = tmp_path / "fpconv_check"
    subprocess.run([cc, "-O2", "-I", CSRC, os.path.join(HERE, "fpconv_check.c"), "-o", str(exe), "-lm"],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 mismatches" in r.stdout
