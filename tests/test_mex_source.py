"""The MATLAB entry point (psd_projection_gb300/matlab/psd_projection_MATLAB.cpp),
compiled and run without MATLAB against a minimal stand-in of the MEX API
(tests/mex_stub/).  It must compile and link against libpsdgb.so (CPU), and
on the GPU give, for every method string of the reference's wrapper
(MATLAB/psd_projection_MATLAB.cu:93-166), the projection within the tolerance
of the other GPU tests (1e-4 relative Frobenius against FP64 dsyevd for the
FP32-class methods, 1e-10 for eig_FP64, and for composite_FP16 1.05x the error
of the oracle's restatement of the reference's FP16 method on the same input)
and the eigenvalues as second output; an unknown method raises the
reference's message.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
SRC = ROOT / "psd_projection_gb300" / "matlab" / "psd_projection_MATLAB.cpp"


def _build(tmp_path):
    from psd_projection_gb300 import _capi

    if not _capi.LIB_PATH.exists():
        pytest.skip("libpsdgb.so is not built")
    exe = tmp_path / "mex_driver"
    cmd = ["g++", "-std=c++17", "-O1", str(SRC), str(HERE / "mex_stub" / "mex_driver.cpp"),
           f"-I{HERE / 'mex_stub'}", f"-I{ROOT / 'include'}", "-o", str(exe), str(_capi.LIB_PATH),
           f"-Wl,-rpath,{_capi.LIB_PATH.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_mex_source_compiles_and_links(tmp_path):
    _build(tmp_path)


@pytest.mark.gpu
@pytest.mark.parametrize("method,tol", [("composite_FP32", 1e-4), ("composite_FP16", None),
                                        ("composite_FP32_emulated", 1e-4), ("eig_FP64", 1e-10),
                                        ("eig_FP32", 1e-4)])
def test_mex_methods(tmp_path, method, tol):
    from oracle import reference_port as rp
    from tests.gpu_util import uniform_spectrum

    exe = _build(tmp_path)
    n = 160
    x = uniform_spectrum(n, 4.0, seed=21)
    np.ascontiguousarray(x.T).tofile(tmp_path / "in.bin")
    args = [str(exe), str(tmp_path / "in.bin"), str(n), method, str(tmp_path / "out.bin")]
    if method.startswith("eig"):
        args.append(str(tmp_path / "eigs.bin"))
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = np.fromfile(tmp_path / "out.bin").reshape(n, n).T
    proj, w = rp.eig_psd(x)
    if tol is None:
        ref, _ = rp.composite_auto_scale(x, "fp16")
        tol = 1.05 * rp.rel_frobenius(ref, proj)
    assert rp.rel_frobenius(out, proj) <= tol
    if method.startswith("eig"):
        eigs = np.fromfile(tmp_path / "eigs.bin")
        assert np.abs(eigs - w).max() <= (1e-10 if method == "eig_FP64" else 1e-5) * np.abs(w).max()


@pytest.mark.gpu
def test_mex_unknown_method(tmp_path):
    exe = _build(tmp_path)
    np.zeros(16).tofile(tmp_path / "in.bin")
    r = subprocess.run([str(exe), str(tmp_path / "in.bin"), "4", "composite_FP8", str(tmp_path / "o.bin")],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 3
    assert "Unknown method. Supported methods: 'composite_FP16'" in r.stdout
