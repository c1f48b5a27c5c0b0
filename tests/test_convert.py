"""The integer-only binary64 -> binary32 narrowing of the copy and split
kernels (psd_projection_gb300/csrc/convert.h), compiled for the host and
compared bit for bit with the host compiler's conversion (CPU only)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_d2f_rn_matches_host_conversion(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "convert_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", str(ROOT / "psd_projection_gb300" / "csrc"),
                    str(ROOT / "tests" / "convert_check.cc"), "-o", str(exe)], check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "0 mismatches" in res.stdout
