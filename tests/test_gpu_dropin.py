"""The C++ drop-in executed: a caller written against the reference's headers
(tests/dropin_caller.cpp) is compiled with g++, linked against libpsdgb.so
and run on the GPU.  It sets a non-default stream on its cuBLAS handle (the
library takes the stream from there), calls the three auto-scaled composite
methods, approximate_two_norm on the reference's 5 x 5 known answer,
eig_FP64_psd / eig_FP32_psd with the eigenvalue array returned for the caller
to free, composite_FP32 with a workspace of the reference's documented size
(3 n^2 floats), and a failing call (printed, then execution continues).

Tolerances (relative Frobenius against the host FP64 dsyevd projection):
1e-4 for the FP32-class methods and eig_FP32_psd; for composite_FP16, 1.05x
the error of the oracle's restatement of the reference's FP16 method on the
same input (test_gpu_configs.py explains the 5 %); 1e-10 for eig_FP64_psd;
the Lanczos bounds must bracket ||A||_2 = 7.0890 as in
test/lanczos_test.hpp:40-41 (up to the rounding of that figure).
"""
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import reference_port as rp
from tests.gpu_util import uniform_spectrum

pytestmark = pytest.mark.gpu
HERE = Path(__file__).resolve().parent
ROOT = HERE.parent


@pytest.fixture(scope="module")
def run_caller(tmp_path_factory):
    from psd_projection_gb300 import _capi
    from psd_projection_gb300 import build as b

    d = tmp_path_factory.mktemp("dropin")
    inputs = {"x300": uniform_spectrum(300, 3.0, seed=11), "x1000": uniform_spectrum(1000, 1.0, seed=12),
              "x1024": uniform_spectrum(1024, 1.0, seed=13),
              "kat5": np.array(json.loads((HERE / "golden" / "kat.json").read_text())["lanczos_two_norm"]["matrix"])}
    for k, v in inputs.items():
        np.ascontiguousarray(np.asarray(v, dtype=np.float64).T).tofile(d / f"{k}.bin")
    cuda_home = Path(b.nvcc()).resolve().parent.parent
    libdir = b.cuda_lib_dir()
    exe = d / "dropin_caller"
    cmd = ["g++", "-std=c++17", "-O1", str(HERE / "dropin_caller.cpp"), f"-I{ROOT / 'include'}",
           f"-I{cuda_home / 'include'}", "-o", str(exe), str(_capi.LIB_PATH), f"-L{libdir}", "-lcublas", "-lcusolver",
           "-lcudart", f"-Wl,-rpath,{_capi.LIB_PATH.parent}", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), str(d)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = {}
    for line in r.stdout.splitlines():
        parts = line.split()
        if parts:
            lines.setdefault(parts[0], []).append(parts[1:])

    class Outputs:
        def __call__(self, name, n):
            return np.fromfile(d / f"{name}.bin", dtype=np.float64).reshape(n, n).T

        def values(self, name):
            return np.fromfile(d / f"{name}.bin", dtype=np.float64)

    return inputs, lines, Outputs(), r.stdout


@pytest.mark.parametrize("method,tol", [("composite_FP32_auto_scale", 1e-4), ("composite_FP16_auto_scale", None),
                                        ("composite_FP32_emulated_auto_scale", 1e-4)])
def test_auto_scaled_methods(run_caller, method, tol):
    inputs, lines, out, _ = run_caller
    proj, _ = rp.eig_psd(inputs["x300"])
    if tol is None:  # the reference FP16 method's own error level on this input
        ref, _ = rp.composite_auto_scale(inputs["x300"], "fp16")
        tol = 1.05 * rp.rel_frobenius(ref, proj)
    assert rp.rel_frobenius(out(method, 300), proj) <= tol


def test_lanczos_kat(run_caller):
    _, lines, _, _ = run_caller
    lo, up = map(float, lines["lanczos"][0])
    two_norm = 7.0890125506
    assert lo <= two_norm * (1 + 1e-9) and two_norm <= up


@pytest.mark.parametrize("which,tol", [("FP64", 1e-10), ("FP32", 1e-4)])
def test_eig_methods_return_caller_freed_eigenvalues(run_caller, which, tol):
    inputs, lines, out, _ = run_caller
    proj, w = rp.eig_psd(inputs["x300"])
    assert rp.rel_frobenius(out(f"eig_{which}_psd", 300), proj) <= tol
    # the unclipped eigenvalues, ascending (src/eig_FP64_psd.cu:30,84)
    got = out.values(f"eig_{which}_values")
    assert np.abs(got - w).max() <= (1e-10 if which == "FP64" else 1e-5) * np.abs(w).max()
    assert "eig_returned_null" not in lines
    assert lines["eig_without_values_null"][0] == ["1"]


def test_reference_sized_workspace(run_caller):
    """3 n^2 floats: used as is when n is a multiple of 128 (no allocation);
    at n = 1000 the padded operands do not fit and the library's own cached
    workspace is allocated instead.  Both results are correct."""
    inputs, lines, out, _ = run_caller
    assert int(lines["workspace_n1024_allocated"][0][0]) == 0
    assert int(lines["workspace_n1000_allocated"][0][0]) > 0
    for n in (1024, 1000):
        proj, _ = rp.eig_psd(inputs[f"x{n}"])
        assert rp.rel_frobenius(out(f"composite_FP32_ws{n}", n), proj) <= 1e-4


def test_failing_call_prints_and_continues(run_caller):
    _, lines, _, stdout = run_caller
    assert "psdgb error 1 in composite_FP32: null matrix" in stdout
    assert lines["continued_after_error"][0] == ["1"]
