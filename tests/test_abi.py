"""The C-ABI library: builds, loads, exports every declared symbol, and the
host-only entry points behave (CPU; no kernel is launched here)."""
import ctypes
import json
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"


@pytest.fixture(scope="module")
def lib():
    from psd_projection_gb300 import _capi, build

    if shutil.which("nvcc") or Path("/usr/local/cuda/bin/nvcc").exists():
        build.build()
    return _capi.lib()


def _exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True, text=True, check=True)
    return {line.split()[-1] for line in out.stdout.splitlines() if " T " in line}


def test_every_header_function_is_exported(lib):
    from psd_projection_gb300 import _capi

    names = _capi.header_functions()
    assert len(names) >= 15
    exported = _exported(_capi.LIB_PATH)
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        getattr(lib, n)


def test_reference_cpp_symbols_are_exported(lib):
    """The mangled C++ entry points of the reference library (built from its
    sources by oracle/build_ref.sh, list in tests/golden/reference_symbols.txt)."""
    from psd_projection_gb300 import _capi

    want = [s for s in (GOLDEN / "reference_symbols.txt").read_text().split() if s]
    assert len(want) >= 9
    built = Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "symbols.txt"
    if built.exists():  # the list is a subset of what the reference build exports
        assert set(want) <= set(built.read_text().split())
    exported = _exported(_capi.LIB_PATH)
    assert set(want) <= exported, sorted(set(want) - exported)


def test_cpp_drop_in_compiles_and_links(lib, tmp_path):
    """Code written against the reference headers compiles against
    include/psd_projection and links against libpsdgb.so unchanged."""
    from psd_projection_gb300 import _capi

    src = tmp_path / "caller.cpp"
    src.write_text(r'''
#include "psd_projection/composite_FP16.h"
#include "psd_projection/composite_FP32.h"
#include "psd_projection/composite_FP32_emulated.h"
#include "psd_projection/eig_FP32_psd.h"
#include "psd_projection/eig_FP64_psd.h"
#include "psd_projection/lanczos.h"
#include "psd_projection/lobpcg.h"
int main(int argc, char**) {
    if (argc > 5) {  // never runs; only the link matters here
        cublasHandle_t h = nullptr; cusolverDnHandle_t s = nullptr; double* m = nullptr; double lo, up;
        composite_FP16(h, m, 8); composite_FP16_auto_scale(h, s, m, 8);
        composite_FP32(h, m, 8); composite_FP32_auto_scale(h, s, m, 8);
        composite_FP32_emulated(h, m, 8); composite_FP32_emulated_auto_scale(h, s, m, 8);
        approximate_two_norm(h, s, m, 8, &lo, &up);
        eig_FP64_psd(s, h, m, 8); eig_FP32_psd(s, h, m, 8, true);
        size_t r = 0;
        compute_eigenpairs(h, s, m, 8, 2, &r, m, m);
        compute_eigenpairs(h, s, m, 8, 0, nullptr, nullptr, nullptr, true, 100, 1e-10, 1e-5);
        composite_FP32_auto_scale_deflate(h, s, m, 8); composite_FP32_auto_scale_deflate(h, s, m, 8, 0, 2);
        composite_FP32_emulated_auto_scale_deflate(h, s, m, 8, 2, 1e-10, 1e-3, false);
        lobpcg(h, s, m, m, m, 6, 2); lobpcg(h, s, m, m, m, 6, 2, 100, 1e-8, true);
        eig_FP64_deflate(s, h, m, 8); eig_FP64_deflate(s, h, m, 8, 2, 50, 1e-8, false);
        composite_FP16_auto_scale_deflate(h, s, m, 8); composite_FP16_auto_scale_deflate(h, s, m, 8, nullptr, nullptr, 2);
    }
    return 0;
}
''')
    cuda_inc = "/usr/local/cuda/include"
    exe = tmp_path / "caller"
    cmd = ["g++", "-std=c++17", str(src), f"-I{ROOT / 'include'}", f"-I{cuda_inc}", "-o", str(exe),
           str(_capi.LIB_PATH), f"-Wl,-rpath,{_capi.LIB_PATH.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_filter_coefficients_match_reference_arithmetic(lib):
    from psd_projection_gb300 import filter_coefficients, SCHEDULE_FP16, SCHEDULE_FP32

    want = json.loads((GOLDEN / "coefficients.json").read_text())
    f32 = ctypes.c_float
    for sched, key in ((SCHEDULE_FP32, "fp32"), (SCHEDULE_FP16, "fp16")):
        got = filter_coefficients(sched)
        assert [[float(f32(v).value) for v in t] for t in got] == want[key]
    assert lib.psdgb_filter_coefficients(7, None, 0) == -1


def test_precision_names_and_workspace(lib):
    from psd_projection_gb300 import PRECISIONS, workspace_size

    for name, code in PRECISIONS.items():
        assert lib.psdgb_precision_name(code).decode() == name
    assert lib.psdgb_precision_name(99) is None
    # three split matrices of Np x Np (Np = n rounded up to 128)
    assert workspace_size(1000, PRECISIONS["fp16x3"]) == 3 * 2 * 2 * 1024 * 1024
    assert workspace_size(1000, PRECISIONS["fp32_simt"]) == 3 * 4 * 1024 * 1024
    assert workspace_size(128, PRECISIONS["bf16x9"]) == 3 * 3 * 2 * 128 * 128
    assert workspace_size(0, PRECISIONS["fp16x3"]) == 0
    assert workspace_size(10, 42) == 0


def test_unknown_method_is_rejected_before_any_device_work(lib):
    from psd_projection_gb300 import _capi

    st = lib.psdgb_project(b"composite_FP8", None, 4, None, None)
    assert st == 1  # PSDGB_ERR_INVALID_ARGUMENT
    assert "Unknown method" in _capi.last_error()
    st = lib.psdgb_project_host(b"nope", None, None, 4, None, None)
    assert st == 1


def test_batch_entry_points_reject_a_null_plan(lib):
    """The batch plan's entry points check their arguments before any device
    work (host logic only)."""
    import ctypes

    vp = ctypes.c_void_p
    for name in ("psdgb_batch_project", "psdgb_batch_project_graph"):
        fn = getattr(lib, name)
        fn.restype = ctypes.c_int
        fn.argtypes = [vp, vp, vp]
        assert fn(None, None, None) == 1, name  # PSDGB_ERR_INVALID_ARGUMENT
    lib.psdgb_batch_destroy.restype = ctypes.c_int
    lib.psdgb_batch_destroy.argtypes = [vp]
    assert lib.psdgb_batch_destroy(None) == 0


def test_version(lib):
    assert lib.psdgb_version() >= 10000
    assert lib.psdgb_kernel_launch_count() == 0 or lib.psdgb_kernel_launch_count() > 0
