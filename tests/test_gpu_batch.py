"""Block-diagonal batch: every block projected as by one call per block (GPU).

Tolerances: batch vs one call per block 1e-5 relative Frobenius per block (the
batch runs each block's Lanczos bound in one CTA with a different reduction
order, so the scale differs in the last bits); each block within 1e-4 of the
FP64 EVD projection (fp16x3).  Graph replay and the autotuned configuration
reproduce the direct launch bit for bit.
"""
import numpy as np
import pytest

from oracle import reference_port as rp
from tests.gpu_util import from_dev, to_dev

pytestmark = pytest.mark.gpu


def _blocks(sizes, seed):
    """(G + G^T)/2 blocks; a 1 x 1 block is kept inside [-1, 1] because the
    reference's Lanczos bound returns up = 1 for n = 1 (its first residual is
    exactly zero), so a larger scalar would leave the filter's interval."""
    rng = np.random.default_rng(seed)
    out = []
    for n in sizes:
        g = rng.standard_normal((n, n))
        m = 0.5 * (g + g.T)
        if n == 1:
            m = np.array([[0.3]])
        out.append(m)
    return out


SIZES = [1, 2, 16, 33, 64, 100, 127, 128, 129, 200, 256, 300, 384, 512, 17, 5, 480, 150, 90, 260]


def test_batch_matches_one_call_per_block():
    import psd_projection_gb300 as psd
    from psd_projection_gb300.batch import BatchPlan, pack, unpack

    mats = _blocks(SIZES, seed=1)
    d = pack(mats)
    with BatchPlan(SIZES) as plan:
        plan.project(d)
        import torch

        torch.cuda.synchronize()
    got = unpack(d, SIZES)
    for n, x, y in zip(SIZES, mats, got):
        t = to_dev(x)
        psd.composite_FP32_auto_scale(t)
        one = from_dev(t)
        assert rp.rel_frobenius(y, one) <= 1e-5 or np.linalg.norm(one) == 0.0, n
        if n >= 2:
            proj, _ = rp.eig_psd(x)
            assert rp.rel_frobenius(y, proj) <= 1e-4, n


def test_batch_large_blocks():
    """Blocks above 512 (up to the 4096 limit) run their Lanczos bound in the
    512-thread class with more than 48 KB of shared memory, next to tiny
    ones; each block matches one call per block."""
    import psd_projection_gb300 as psd
    from psd_projection_gb300.batch import BatchPlan, pack, unpack

    sizes = [700, 20, 1030, 3]
    mats = _blocks(sizes, seed=4)
    d = pack(mats)
    with BatchPlan(sizes) as plan:
        plan.project(d)
        import torch

        torch.cuda.synchronize()
    got = unpack(d, sizes)
    for n, x, y in zip(sizes, mats, got):
        t = to_dev(x)
        psd.composite_FP32_auto_scale(t)
        assert rp.rel_frobenius(y, from_dev(t)) <= 1e-5, n


def test_batch_graph_replay_and_autotune():
    import torch

    from psd_projection_gb300.batch import BatchPlan, pack, unpack

    sizes = SIZES * 3
    mats = _blocks(sizes, seed=2)
    pristine = pack(mats)
    with BatchPlan(sizes) as plan:
        direct = pristine.clone()
        plan.project(direct)
        torch.cuda.synchronize()
        scratch = pristine.clone()
        plan.autotune(scratch)
        tuned = pristine.clone()
        plan.project(tuned)
        work = pristine.clone()
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            plan.project(work.clone(), stream=side)
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        with torch.cuda.graph(g):
            plan.project(work)
        work.copy_(pristine)
        g.replay()
        torch.cuda.synchronize()
        info = plan.info()
    a, b, c = unpack(direct, sizes), unpack(tuned, sizes), unpack(work, sizes)
    for x, y, z in zip(a, b, c):
        assert np.array_equal(y, z)
        assert rp.rel_frobenius(x, y) <= 1e-6 or np.linalg.norm(x) == 0.0
    assert info["num_tiles"] > 0


def test_batch_bf16x9_and_fp16():
    import psd_projection_gb300 as psd
    from psd_projection_gb300.batch import BatchPlan, pack, unpack

    sizes = [64, 200, 130]
    mats = _blocks(sizes, seed=3)
    for prec, sched, tol in ((psd.PRECISIONS["bf16x9"], psd.SCHEDULE_FP32, 1e-4),
                             (psd.PRECISIONS["fp16"], psd.SCHEDULE_FP16, 2e-3)):
        d = pack(mats)
        with BatchPlan(sizes, prec, sched) as plan:
            plan.project(d)
        got = unpack(d, sizes)
        for x, y in zip(mats, got):
            proj, _ = rp.eig_psd(x)
            assert rp.rel_frobenius(y, proj) <= tol


# Blocks of every size class around the 64 / 128 boundaries of the on-chip
# route (one or two K blocks, one tile), an empty block, and larger blocks.
ON_CHIP_SIZES = [0, 1, 2, 16, 33, 63, 64, 65, 100, 127, 128, 129, 200, 300, 5, 90, 256, 17]


@pytest.mark.parametrize("prec_name,sched_name", [("fp16x3", "SCHEDULE_FP32"), ("fp16", "SCHEDULE_FP16")])
def test_batch_small_blocks_on_chip_bit_identical(prec_name, sched_name):
    """The on-chip route for blocks of n <= 128 (one persistent kernel, the
    split matrices in shared memory) and the per-product launches give the
    same result bit for bit with one accumulator per tile, in both tile
    orders; each block within 1e-4 (fp16x3) / 2e-3 (fp16) of FP64 EVD."""
    import torch

    import psd_projection_gb300 as psd
    from psd_projection_gb300.batch import BatchPlan, pack, unpack

    mats = _blocks(ON_CHIP_SIZES, seed=7)
    pristine = pack(mats)
    outs = {}
    with BatchPlan(ON_CHIP_SIZES, psd.PRECISIONS[prec_name], getattr(psd, sched_name)) as plan:
        t = plan.tuning()
        assert t["small_blocks"] == sum(1 for n in ON_CHIP_SIZES if 1 <= n <= 128)
        assert t["small_on_chip"] == 1
        for order in (0, 1):
            for chip in (1, 0):
                plan.configure(acc_mode=2, tile_order=order, small_on_chip=chip)
                d = pristine.clone()
                plan.project(d)
                torch.cuda.synchronize()
                outs[(order, chip)] = d.cpu().numpy()
    ref = outs[(0, 0)]
    for key, v in outs.items():
        assert np.array_equal(v, ref), key
    tol = 1e-4 if prec_name == "fp16x3" else 2e-3
    for n, x, y in zip(ON_CHIP_SIZES, mats, unpack(torch.from_numpy(ref), ON_CHIP_SIZES)):
        if n >= 2:
            proj, _ = rp.eig_psd(x)
            assert rp.rel_frobenius(y, proj) <= tol, n


def test_batch_only_small_blocks_and_graph():
    """A batch of small blocks only (nothing left for the per-product
    launches) on the on-chip route, direct and replayed from a CUDA graph."""
    import torch

    import psd_projection_gb300 as psd
    from psd_projection_gb300.batch import BatchPlan, pack, unpack

    sizes = [1, 7, 64, 65, 128, 100, 40] * 40
    mats = _blocks(sizes, seed=8)
    pristine = pack(mats)
    with BatchPlan(sizes) as plan:
        assert plan.tuning()["small_on_chip"] == 1
        direct = pristine.clone()
        plan.project(direct)
        work = pristine.clone()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            plan.project(work.clone(), stream=side)
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            plan.project(work)
        work.copy_(pristine)
        g.replay()
        torch.cuda.synchronize()
    assert torch.equal(direct, work)
    for n, x, y in zip(sizes[:7], mats[:7], unpack(direct, sizes)[:7]):
        t = to_dev(x)
        psd.composite_FP32_auto_scale(t)
        assert rp.rel_frobenius(y, from_dev(t)) <= 1e-5 or np.linalg.norm(y) == 0.0, n


def test_batch_on_chip_refused_without_fp16_pairs():
    import psd_projection_gb300 as psd
    from psd_projection_gb300.batch import BatchPlan

    with BatchPlan([64, 200], psd.PRECISIONS["bf16x9"], psd.SCHEDULE_FP32) as plan:
        assert plan.tuning()["small_on_chip"] == 0
        with pytest.raises(psd.PsdgbError, match="on chip"):
            plan.configure(small_on_chip=1)
        plan.configure(acc_mode=1, tile_order=1, small_on_chip=0)
        t = plan.tuning()
        assert (t["acc_mode"], t["tile_order"]) == (1, 1)


@pytest.mark.parametrize("prec_name,sched_name", [("fp16x3", "SCHEDULE_FP32"), ("bf16x9", "SCHEDULE_FP32")])
def test_batch_pair_tiles_match_single_tiles(prec_name, sched_name):
    """Blocks of n > 128 on 256 x 256 pair tiles (the odd last tile row of a
    block on 128 x 128 tiles) against 128 x 128 tiles only, one accumulator
    per tile: the same term products in the same K order, but a 256-wide MMA
    on a CTA pair and a 128-wide one do not round their internal sums alike
    (measured: 1.1-1.6e-6 relative apart at n = 600, below 1e-6 up to
    n = 512), so the two agree to 5e-6 relative per block, below the
    filter's own error against FP64 EVD (about 5e-6), and each shape gives
    the same bits in both tile orders.  Each block within 1e-4 of FP64 EVD.
    Sizes cover one, two, three, four and five tile rows."""
    import torch

    import psd_projection_gb300 as psd
    from psd_projection_gb300.batch import BatchPlan, pack, unpack

    sizes = [129, 200, 256, 257, 300, 384, 385, 512, 600, 640, 40, 100, 1, 0]
    mats = _blocks(sizes, seed=9)
    pristine = pack(mats)
    outs = {}
    with BatchPlan(sizes, psd.PRECISIONS[prec_name], getattr(psd, sched_name)) as plan:
        t = plan.tuning()
        # pair tiles per block: np 256 -> 1, 384 -> 1, 512 -> 3, 640 -> 3
        assert t["pair_tiles"] == 0 and t["num_pair_tiles"] == 3 * 1 + 3 * 1 + 2 * 3 + 2 * 3
        for order in (0, 1):
            for pairs in (1, 0):
                plan.configure(acc_mode=2, tile_order=order, pair_tiles=pairs)
                d = pristine.clone()
                plan.project(d)
                torch.cuda.synchronize()
                outs[(order, pairs)] = d.cpu().numpy()
    for pairs in (0, 1):
        assert np.array_equal(outs[(0, pairs)], outs[(1, pairs)]), pairs
    single = unpack(torch.from_numpy(outs[(0, 0)]), sizes)
    paired = unpack(torch.from_numpy(outs[(0, 1)]), sizes)
    for n, x, y0, y1 in zip(sizes, mats, single, paired):
        if n >= 2:
            proj, _ = rp.eig_psd(x)
            assert rp.rel_frobenius(y0, proj) <= 1e-4, n
            assert rp.rel_frobenius(y1, proj) <= 1e-4, n
            d = rp.rel_frobenius(y1, y0)
            assert d <= 5e-6, (n, d)


def test_batch_serpentine_order_same_bits():
    """Every other product walking its tile lists backwards changes the order
    in which tiles run, not what any tile computes: the same bits, for both
    tile shapes."""
    import torch

    from psd_projection_gb300.batch import BatchPlan, pack

    sizes = [300, 40, 512, 129, 256, 90, 385]
    mats = _blocks(sizes, seed=10)
    pristine = pack(mats)
    outs = []
    with BatchPlan(sizes) as plan:
        for pairs in (0, 1):
            for serp in (0, 1):
                plan.configure(pair_tiles=pairs, serpentine=serp)
                assert plan.tuning()["serpentine"] == serp
                d = pristine.clone()
                plan.project(d)
                torch.cuda.synchronize()
                outs.append((pairs, serp, d.cpu().numpy()))
    for pairs, serp, v in outs:
        ref = next(w for p, s, w in outs if p == pairs and s == 0)
        assert np.array_equal(v, ref), (pairs, serp)


def test_batch_plan_graph_same_bits():
    """psdgb_batch_project_graph (the plan's own graph, stream priorities
    kept) reproduces psdgb_batch_project bit for bit: on first capture, on
    replay, after a configuration change and for another blocks pointer."""
    import torch

    from psd_projection_gb300.batch import BatchPlan, pack

    sizes = [300, 40, 512, 129, 256, 90, 385, 16]
    mats = _blocks(sizes, seed=13)
    pristine = pack(mats)
    with BatchPlan(sizes) as plan:
        ref = pristine.clone()
        plan.project(ref)
        torch.cuda.synchronize()
        ref = ref.cpu().numpy()
        d = pristine.clone()
        for _ in range(3):  # capture, then two replays on restored input
            d.copy_(pristine)
            plan.project_graph(d)
            torch.cuda.synchronize()
            assert np.array_equal(d.cpu().numpy(), ref)
        other = pristine.clone()  # a new pointer: captured again
        plan.project_graph(other)
        torch.cuda.synchronize()
        assert np.array_equal(other.cpu().numpy(), ref)
        for chip in (0, 1):  # a new configuration: captured again, same bits (acc_mode 2)
            plan.configure(acc_mode=2, small_on_chip=chip)
            d.copy_(pristine)
            plan.project_graph(d)
            torch.cuda.synchronize()
            r = pristine.clone()
            plan.project(r)
            torch.cuda.synchronize()
            assert np.array_equal(d.cpu().numpy(), r.cpu().numpy()), chip
