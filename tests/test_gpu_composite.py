"""Composite filter on the GPU: the reference's KATs and bars, parity with the
oracle restatement and with the model of the kernels' arithmetic, edge cases.

Tolerances (relative Frobenius unless stated):
  * against FP64 EVD: 1e-4 for the FP32-class precisions (fp32_simt, fp16x3,
    bf16x6, bf16x9, bf16x3) — the spec bar; 1e-3 for fp16 (the
    reference's FP16 bar, test/composite_FP16_test.hpp:129); 1e-2 for bf16
    (a one-term mode the reference does not have, reported not targeted);
  * GPU against the split-arithmetic model on the same input: 3e-5 for
    fp32_simt / fp16x3 / bf16x6 / bf16x9 and 1e-4 for bf16x3 — the model
    accumulates in FP64 where the tensor cores accumulate in FP32; 1e-2 (fp16)
    and 5e-2 (bf16) for the one-term modes, whose 11 / 8-bit operand rounding
    turns a last-bit accumulator difference into an operand-rounding flip;
  * the reference's own bars: rel <= 1e-3 (test/composite_FP32_test.hpp:121),
    abs <= 0.1 at lambda in [-10, 10] (:191, :239), KAT elementwise 1e-3 (:76);
    the reference asserts its KATs on the FP32 path only, so the one-term
    modes are held to 1e-2 (fp16) and 3e-2 (bf16) there.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import reference_port as rp
from tests.gpu_util import from_dev, gaussian_sym, to_dev, uniform_spectrum

pytestmark = pytest.mark.gpu
KAT = json.loads((Path(__file__).resolve().parent / "golden" / "kat.json").read_text())

FP32_CLASS = ["fp32_simt", "fp16x3", "bf16x3", "bf16x6", "bf16x9"]
ALL = FP32_CLASS + ["fp16", "bf16"]
EVD_TOL = {"fp16": 1e-3, "bf16": 1e-2}
MODEL_TOL = {"fp16": 1e-2, "bf16": 5e-2, "bf16x3": 1e-4}
KAT_TOL = {"fp16": 1e-2, "bf16": 3e-2}


def sched(p):
    return "fp16" if p in ("fp16", "bf16") else "fp32"


@pytest.fixture(scope="module")
def psd():
    import psd_projection_gb300 as psd

    return psd


def run(psd, x, precision, auto_scale, **kw):
    t = to_dev(x)
    code = psd.PRECISIONS[precision]
    s = psd.SCHEDULE_FP16 if sched(precision) == "fp16" else psd.SCHEDULE_FP32
    up = psd.composite(t, code, s, auto_scale=auto_scale, **kw)
    return from_dev(t), up


@pytest.mark.parametrize("precision", ALL)
def test_kat_deterministic(psd, precision):
    k = KAT["composite_fp32_deterministic"]
    x = np.array(k["input_over_15"]) / 15.0
    out, _ = run(psd, x, precision, auto_scale=False)
    assert np.abs(out - np.array(k["expected"])).max() <= KAT_TOL.get(precision, k["tolerance"])


@pytest.mark.parametrize("precision", ALL)
def test_kat_simple5(psd, precision):
    k = KAT["composite_simple5"]
    out, _ = run(psd, np.diag(k["diagonal"]), precision, auto_scale=True)
    assert np.abs(out - np.diag(k["expected_diagonal"])).max() <= KAT_TOL.get(precision, k["tolerance"])


@pytest.mark.parametrize("precision", ALL)
def test_bar_uniform_scaled(psd, precision):
    """UniformScaled: n = 1000, spectrum [-1, 1], no scaling."""
    x = uniform_spectrum(1000, 1.0, seed=1)
    proj, _ = rp.eig_psd(x)
    out, _ = run(psd, x, precision, auto_scale=False)
    err = rp.rel_frobenius(out, proj)
    assert err <= 1e-3 or precision == "bf16"
    assert err <= EVD_TOL.get(precision, 1e-4), err


@pytest.mark.parametrize("precision", FP32_CLASS + ["fp16"])
def test_bar_autoscaled_abs(psd, precision):
    """UniformAutoScaled1024: n = 1024, spectrum [-10, 10], Lanczos scaling."""
    x = uniform_spectrum(1024, 10.0, seed=2)
    proj, _ = rp.eig_psd(x)
    out, up = run(psd, x, precision, auto_scale=True)
    assert np.linalg.norm(out - proj) <= (0.1 if precision != "fp16" else 0.5)
    assert up >= np.linalg.norm(x, 2)


@pytest.mark.parametrize("precision", ALL)
@pytest.mark.parametrize("n", [3, 17, 100, 129])
def test_parity_with_kernel_model(psd, precision, n):
    x = gaussian_sym(n, seed=n)
    x = x / np.linalg.norm(x, 2)
    out, _ = run(psd, x, precision, auto_scale=False)
    model = rp.composite_split_model(x, precision, sched(precision))
    assert rp.rel_frobenius(out, model) <= MODEL_TOL.get(precision, 3e-5)


@pytest.mark.parametrize("precision", FP32_CLASS)
def test_parity_with_reference_restatement(psd, precision):
    """GPU FP32-class result against the FP32 restatement of composite_FP32
    on the committed golden cases."""
    g = np.load(Path(__file__).resolve().parent / "golden" / "cases.npz")
    for n in (16, 64, 100):
        out, _ = run(psd, g[f"x_{n}"], precision, auto_scale=False)
        assert rp.rel_frobenius(out, g[f"fp32_{n}"]) <= 3e-5
        assert rp.rel_frobenius(out, g[f"evd_{n}"]) <= 1e-4


@pytest.mark.parametrize("precision", ["fp16x3", "fp32_simt"])
def test_autoscale_parity_with_oracle(psd, precision):
    x = gaussian_sym(300, seed=7)
    out, up = run(psd, x, precision, auto_scale=True)
    want, up_ref = rp.composite_auto_scale(x.astype(np.float32).astype(np.float64))
    assert up == pytest.approx(up_ref, rel=1e-4)
    assert rp.rel_frobenius(out, want) <= 3e-5
    proj, _ = rp.eig_psd(x)
    assert rp.rel_frobenius(out, proj) <= 1e-4


def test_bf16_one_term_requires_fp16_schedule(psd):
    t = to_dev(np.eye(8) * 0.5)
    with pytest.raises(psd.PsdgbError, match="FP16 schedule"):
        psd.composite(t, psd.PRECISIONS["bf16"], psd.SCHEDULE_FP32, auto_scale=False)


def test_empty_and_tiny(psd):
    import torch

    t = torch.zeros((0, 0), dtype=torch.float64, device="cuda")
    assert psd.composite(t) == 1.0
    for v in (0.5, -0.5, 0.0):
        out, _ = run(psd, np.array([[v]]), "fp16x3", auto_scale=False)
        assert out[0, 0] == pytest.approx(max(v, 0.0), abs=2e-3)
    out, _ = run(psd, np.array([[0.3, 0.4], [0.4, -0.3]]), "fp16x3", auto_scale=True)
    proj, _ = rp.eig_psd(np.array([[0.3, 0.4], [0.4, -0.3]]))
    assert np.abs(out - proj).max() <= 1e-4


def test_nonsymmetric_input_uses_upper_triangle(psd):
    x = np.random.default_rng(5).standard_normal((77, 77)) * 0.05
    a, _ = run(psd, x, "fp16x3", auto_scale=True)
    b, _ = run(psd, rp.sym_upper(x), "fp16x3", auto_scale=True)
    assert np.array_equal(a, b)
    assert np.array_equal(a, a.T)


@pytest.mark.parametrize("precision", ["fp16x3", "bf16x9", "fp16"])
def test_deterministic_and_workspace(psd, precision):
    import torch

    x = gaussian_sym(200, seed=11)
    a, _ = run(psd, x, precision, auto_scale=True)
    b, _ = run(psd, x, precision, auto_scale=True)
    assert np.array_equal(a, b)
    ws = torch.empty(psd.workspace_size(200, psd.PRECISIONS[precision]), dtype=torch.uint8, device="cuda")
    c, _ = run(psd, x, precision, auto_scale=True, workspace=ws)
    assert np.array_equal(a, c)


def test_unaligned_workspace_is_refused(psd):
    """A caller workspace that is not 16-byte aligned (TMA tensor maps and
    16-byte vector stores read and write it) gives an invalid-argument error
    before anything runs; the matrix is untouched."""
    import torch

    x = gaussian_sym(200, seed=13)
    ws = torch.empty(psd.workspace_size(200, psd.PRECISIONS["fp16x3"]) + 64, dtype=torch.uint8, device="cuda")
    t = to_dev(x)
    with pytest.raises(psd.PsdgbError) as e:
        psd.composite(t, psd.PRECISIONS["fp16x3"], psd.SCHEDULE_FP32, auto_scale=True, workspace=ws[4:])
    assert e.value.status == 1 and "aligned" in str(e.value)
    assert np.array_equal(from_dev(t), x)


def test_reference_method_mapping(psd):
    """composite_FP32 / _FP16 / _emulated entry points use fp16x3 / fp16 / bf16x9."""
    x = uniform_spectrum(150, 1.0, seed=12)
    proj, _ = rp.eig_psd(x)
    for fn, tol in ((psd.composite_FP32, 1e-4), (psd.composite_FP32_emulated, 1e-4), (psd.composite_FP16, 1.5e-3)):
        t = to_dev(x)
        fn(t)
        assert rp.rel_frobenius(from_dev(t), proj) <= tol
    for fn, tol in ((psd.composite_FP32_auto_scale, 1e-4), (psd.composite_FP32_emulated_auto_scale, 1e-4),
                    (psd.composite_FP16_auto_scale, 2e-3)):
        t = to_dev(x * 7.0)
        fn(t)
        assert rp.rel_frobenius(from_dev(t), proj * 7.0) <= tol


def _async_buffers(psd, n, precision, max_iter=20):
    import torch

    lib = psd._capi.lib()
    ws = torch.empty(psd.workspace_size(n, precision), dtype=torch.uint8, device="cuda")
    lz = torch.empty(lib.psdgb_lanczos_state_size(n, max_iter), dtype=torch.uint8, device="cuda")
    return ws, lz


def _run_async(psd, t, precision, ws, lz, warm=None, ritz=None, stream=None, max_iter=20):
    import ctypes

    import torch

    lib = psd._capi.lib()
    n = t.shape[0]
    s = stream if stream is not None else torch.cuda.current_stream()
    st = lib.psdgb_composite_auto_scale_async(
        precision, psd.SCHEDULE_FP32, ctypes.c_void_p(t.data_ptr()), n, max_iter, 1e-10, psd.DEFAULT_SEED, 0,
        ctypes.c_void_p(warm.data_ptr()) if warm is not None else None,
        ctypes.c_void_p(ritz.data_ptr()) if ritz is not None else None,
        ctypes.c_void_p(ws.data_ptr()), ws.numel(), ctypes.c_void_p(lz.data_ptr()), lz.numel(),
        ctypes.c_void_p(s.cuda_stream))
    psd._capi.check(st, "psdgb_composite_auto_scale_async")


def test_async_matches_sync_and_warm_start(psd):
    import torch

    prec = psd.PRECISIONS["fp16x3"]
    x = gaussian_sym(260, seed=21)
    want, _ = run(psd, x, "fp16x3", auto_scale=True)
    ws, lz = _async_buffers(psd, 260, prec)
    t = to_dev(x)
    ritz = torch.empty(260, dtype=torch.float64, device="cuda")
    _run_async(psd, t, prec, ws, lz, ritz=ritz)
    torch.cuda.synchronize()
    assert psd._capi.lib().psdgb_check_device_error() == 0
    assert np.array_equal(from_dev(t), want)
    # ADMM-style repeat call: a slightly changed matrix, warm-started from the previous Ritz vector.
    e = np.random.default_rng(22).standard_normal((260, 260))
    x2 = x + 1e-2 * 0.5 * (e + e.T)
    t2 = to_dev(x2)
    _run_async(psd, t2, prec, ws, lz, warm=ritz, max_iter=20)
    torch.cuda.synchronize()
    proj2, _ = rp.eig_psd(x2)
    assert rp.rel_frobenius(from_dev(t2), proj2) <= 1e-4


def test_async_path_captures_in_a_cuda_graph(psd):
    import torch

    prec = psd.PRECISIONS["fp16x3"]
    n = 300
    x = gaussian_sym(n, seed=23)
    want, _ = run(psd, x, "fp16x3", auto_scale=True)
    ws, lz = _async_buffers(psd, n, prec)
    static_in = to_dev(np.zeros((n, n)))
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):  # warm-up outside capture
        _run_async(psd, static_in, prec, ws, lz, stream=side)
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        _run_async(psd, static_in, prec, ws, lz)
    for _ in range(2):
        static_in.copy_(to_dev(x))
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(from_dev(static_in), want)


def test_mixed_bulk_and_refinement(psd):
    """Low-precision bulk + split-precision refinement: valid and bounded."""
    x = uniform_spectrum(300, 3.0, seed=31)
    proj, _ = rp.eig_psd(x)
    t = to_dev(x)
    psd.composite_mixed(t, "fp16", "fp16x3", 2)
    assert rp.rel_frobenius(from_dev(t), proj) <= 3e-3
    t = to_dev(x)
    psd.composite_mixed(t, "bf16", "bf16x9", 1)
    assert rp.rel_frobenius(from_dev(t), proj) <= 3e-2
    with pytest.raises(psd.PsdgbError, match="operand format"):
        psd.composite_mixed(to_dev(x), "fp16", "bf16x9", 1)


@pytest.mark.parametrize("precision", ["fp16x3", "bf16x9", "fp16", "bf16x6"])
@pytest.mark.parametrize("n", [129, 300, 513, 1000])
@pytest.mark.parametrize("acc_mode", [0, 1, 2])
def test_pair_products_match_single_cta(psd, precision, n, acc_mode):
    """Products on CTA pairs (256 x 128 tiles, one cta_group::2 MMA over two
    SMs) and products with one CTA per 128 x 128 tile give the same projection
    (same term products, same K order per accumulator): relative difference
    <= 1e-6, and each within the FP32-class bar of the FP64 EVD projection."""
    x = uniform_spectrum(n, 2.0, seed=40 + n)
    proj, _ = rp.eig_psd(x)
    prev_acc = psd.set_product_config(acc_mode)
    prev_shape = psd.set_product_tuning(psd.TUNE_TILE_SHAPE, psd.TILE_128X128)
    try:
        single, _ = run(psd, x, precision, auto_scale=True)
        psd.set_product_tuning(psd.TUNE_TILE_SHAPE, psd.TILE_PAIR_256X128)
        pair, _ = run(psd, x, precision, auto_scale=True)
    finally:
        psd.set_product_tuning(psd.TUNE_TILE_SHAPE, prev_shape)
        psd.set_product_config(prev_acc)
    assert np.linalg.norm(pair - single) <= 1e-6 * np.linalg.norm(single)
    bar = 2e-3 if precision == "fp16" else 1e-4
    assert rp.rel_frobenius(pair, proj) <= bar


@pytest.mark.parametrize("group", [0, 1, 3, 8])
def test_tile_order_does_not_change_results(psd, group):
    """The tile order (grouped raster) changes which CTA computes a tile, not its arithmetic: bit-identical."""
    x = uniform_spectrum(700, 1.5, seed=77)
    prev = psd.set_product_tuning(psd.TUNE_TILE_GROUP, 0)
    try:
        ref, _ = run(psd, x, "fp16x3", auto_scale=True)
        psd.set_product_tuning(psd.TUNE_TILE_GROUP, group)
        got, _ = run(psd, x, "fp16x3", auto_scale=True)
    finally:
        psd.set_product_tuning(psd.TUNE_TILE_GROUP, prev)
    assert np.array_equal(ref, got)


@pytest.mark.parametrize("precision", ["fp16x3", "bf16x3", "fp16", "bf16"])
@pytest.mark.parametrize("n", [129, 300, 513, 1000])
def test_wide_tiles_match_oracle(psd, precision, n):
    """128 x 256 tiles: within the bars of the FP64 EVD projection and close
    to the 128 x 128 kernel.  The K order per accumulator differs, so the two
    differ by about the precision's own error: <= 1e-5 for fp16x3, 5e-5 for
    bf16x3 (1.8e-5 from the exact projection at n = 8192), 1e-3 for the
    one-term products."""
    x = uniform_spectrum(n, 2.0, seed=60 + n)
    proj, _ = rp.eig_psd(x)
    prev_shape = psd.set_product_tuning(psd.TUNE_TILE_SHAPE, psd.TILE_128X128)
    try:
        ref, _ = run(psd, x, precision, auto_scale=True)
        psd.set_product_tuning(psd.TUNE_TILE_SHAPE, psd.TILE_WIDE_128X256)
        wide, _ = run(psd, x, precision, auto_scale=True)
    finally:
        psd.set_product_tuning(psd.TUNE_TILE_SHAPE, prev_shape)
    one_term = precision in ("fp16", "bf16")
    diff_tol = {"fp16x3": 1e-5, "bf16x3": 5e-5}.get(precision, 1e-3)
    assert np.linalg.norm(wide - ref) <= diff_tol * np.linalg.norm(ref)
    assert rp.rel_frobenius(wide, proj) <= EVD_TOL.get(precision, 1e-4) * (2 if one_term else 1)


@pytest.mark.parametrize("precision", ["fp16x3", "bf16x3", "fp16"])
def test_default_large_path_matches_evd(psd, precision):
    """n = 2100 takes the automatic large-matrix path (128 x 256 tiles, K in
    register-summed chunks): within the bars of the FP64 EVD projection, and
    the 32- and 64-wide K blocks agree."""
    x = uniform_spectrum(2100, 1.0, seed=9)
    proj, _ = rp.eig_psd(x)
    out, _ = run(psd, x, precision, auto_scale=True)
    # One-term FP16 products lose accuracy with n (1.4e-3 here, 1.25e-3 at
    # n = 8192, on either tile shape): its bar at this size is 2e-3.
    assert rp.rel_frobenius(out, proj) <= (2e-3 if precision == "fp16" else 1e-4)
    prev = psd.set_product_tuning(psd.TUNE_WIDE_KBLOCK, 64 if precision != "fp16" else 32)
    try:
        other, _ = run(psd, x, precision, auto_scale=True)
    finally:
        psd.set_product_tuning(psd.TUNE_WIDE_KBLOCK, prev)
    assert np.linalg.norm(other - out) <= (1e-3 if precision == "fp16" else 2e-5) * np.linalg.norm(out)


@pytest.mark.parametrize("precision", ["fp16x3", "fp16"])
@pytest.mark.parametrize("n", [300, 2100])
def test_f32_io_matches_f64_path(psd, precision, n):
    """FP32 in / FP32 out (psdgb_composite_auto_scale_f32) on an input exact in
    FP32: the same bound, filter and reconstruction as the FP64 path, whose
    result it returns rounded to FP32 (rel. difference <= 3e-7); the lower
    triangle is ignored (upper-triangle semantics, as the FP64 path)."""
    import torch

    x = uniform_spectrum(n, 3.0, seed=70 + n).astype(np.float32).astype(np.float64)
    ref, _ = run(psd, x, precision, auto_scale=True)
    garbage = np.triu(x) + np.tril(np.full_like(x, 7.0), -1)  # column-major upper triangle = row-major lower
    t = torch.from_numpy(np.ascontiguousarray(garbage.T).astype(np.float32)).cuda()
    s = psd.SCHEDULE_FP16 if precision == "fp16" else psd.SCHEDULE_FP32
    psd.composite_f32(t, psd.PRECISIONS[precision], s)
    torch.cuda.synchronize()
    assert psd._capi.lib().psdgb_check_device_error() == 0
    out = t.cpu().numpy().T.astype(np.float64)
    assert np.linalg.norm(out - ref) <= 3e-7 * np.linalg.norm(ref)


def test_f32_io_warm_start(psd):
    import torch

    n = 400
    x = uniform_spectrum(n, 2.0, seed=81).astype(np.float32)
    ritz = torch.empty(n, dtype=torch.float64, device="cuda")
    t = torch.from_numpy(x).cuda()
    psd.composite_f32(t, ritz_out=ritz)
    e = np.random.default_rng(82).standard_normal((n, n)).astype(np.float32)
    x2 = x + 1e-2 * 0.5 * (e + e.T)
    t2 = torch.from_numpy(x2).cuda()
    psd.composite_f32(t2, warm_start=ritz, max_iter=10)
    torch.cuda.synchronize()
    proj, _ = rp.eig_psd(x2.astype(np.float64))
    assert rp.rel_frobenius(t2.cpu().numpy().astype(np.float64), proj) <= 1e-4
    with pytest.raises(TypeError):
        psd.composite_f32(torch.zeros((4, 4), dtype=torch.float64, device="cuda"))
    with pytest.raises(psd.PsdgbError, match="tensor-core"):
        psd.composite_f32(torch.zeros((4, 4), dtype=torch.float32, device="cuda"), psd.PRECISIONS["fp32_simt"])


@pytest.mark.parametrize("precision", ["fp16x3", "bf16x3", "fp16"])
@pytest.mark.parametrize("n", [300, 513, 1000, 2100])
def test_pair_wide_tiles_match_wide(psd, precision, n):
    """256 x 256 tiles on CTA pairs (one cta_group::2 MMA of 256 x 256 x 16
    over two SMs) against 128 x 256 tiles on one CTA: the same term products
    and K chunks, so the same projection (relative difference <= 1e-6), within
    the bars of the FP64 EVD projection."""
    x = uniform_spectrum(n, 2.0, seed=90 + n)
    proj, _ = rp.eig_psd(x)
    prev = psd.set_product_tuning(psd.TUNE_TILE_SHAPE, psd.TILE_WIDE_128X256)
    try:
        wide, _ = run(psd, x, precision, auto_scale=True)
        psd.set_product_tuning(psd.TUNE_TILE_SHAPE, psd.TILE_PAIR_256X256)
        pair, _ = run(psd, x, precision, auto_scale=True)
    finally:
        psd.set_product_tuning(psd.TUNE_TILE_SHAPE, prev)
    assert np.linalg.norm(pair - wide) <= 1e-6 * np.linalg.norm(wide)
    assert rp.rel_frobenius(pair, proj) <= (2e-3 if precision == "fp16" else 1e-4)


@pytest.mark.parametrize("precision", ["bf16x9", "bf16x6"])
@pytest.mark.parametrize("n", [300, 2100])
def test_three_term_pair_tiles_match_single_cta_tiles(psd, precision, n):
    """Three-term BF16 products on 256 x 256 pair tiles (32-wide K blocks, K
    summed in register chunks of 1024 — the default from n = 2048) against
    the 128 x 128 single-CTA kernel: both within the FP32-class bar of the FP64
    EVD projection, and within 1e-5 of each other (the K summation order
    differs)."""
    x = uniform_spectrum(n, 2.0, seed=80 + n)
    proj, _ = rp.eig_psd(x)
    prev_shape = psd.set_product_tuning(psd.TUNE_TILE_SHAPE, psd.TILE_128X128)
    try:
        single, _ = run(psd, x, precision, auto_scale=True)
        psd.set_product_tuning(psd.TUNE_TILE_SHAPE, psd.TILE_PAIR_256X256)
        pair, _ = run(psd, x, precision, auto_scale=True)
    finally:
        psd.set_product_tuning(psd.TUNE_TILE_SHAPE, prev_shape)
    assert rp.rel_frobenius(single, proj) <= 1e-4
    assert rp.rel_frobenius(pair, proj) <= 1e-4
    assert np.linalg.norm(pair - single) <= 1e-5 * np.linalg.norm(single)
