#!/usr/bin/env python
"""bench.py — throughput of the GB300 PSD projection on the n = 8192 workload.

Workload (one "step" = one auto-scaled projection of one matrix):
  n = 8192, A = Q diag(lambda) Q^T with Q from the QR of a seeded N(0, 1)
  matrix and lambda ~ U[-1, 1] (seeded), symmetrised and stored in FP32, passed
  as the FP64 column-major matrix the reference's API takes.  The exact
  projection Q diag(max(lambda, 0)) Q^T is the FP64 oracle every result's
  relative Frobenius error is quoted against.

Arms:
  (default)          this library: composite_FP32_auto_scale through the C ABI
                     (Lanczos bound + 10-step filter on fp16x3 tensor-core
                     products + fused ReLU reconstruction), inputs resident in
                     HBM (one 537 MB input per step, more than L2, no flush);
                     `e2e` runs psdgb_project_host_many("composite_FP32") on pinned
                     host buffers with both copies inside the timed region.
  --impl reference   the reference's CPU path named by the goal: FP64 LAPACK
                     dsyevd EVD projection (eig_FP64_psd's math) of the full
                     n = 8192 matrix on all host cores, one per step; plus the
                     reference's three GPU methods (composite_FP32 on FP32
                     Sgemm, composite_FP16 on FP16 GemmEx, composite_FP32_emulated
                     on cuBLAS's BF16x9 emulation, each auto-scaled) replayed
                     call for call on cuBLAS / cuSOLVER, with the reference's
                     per-call allocation and with caller workspaces.

Multi-GPU: a single projection does not shard, so N GPUs run N independent
replicas (one process per GPU under torchrun) and `value` is N x steps over
the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "n=8192 proj/s & TC TFLOP/s vs plain FP32 at equal error; p50/p99 serve latency"

# DRAM bytes (read + write) of one product launch, from one ncu capture of the
# same kernel on the same workload size (profiles/ holds the summary).
TRAFFIC_PER_LAUNCH = {(8192, "fp16x3", True): 1.72e9}
TRAFFIC_SOURCE = "ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch (profiles/tc_pairwide_kernel_fp16x3_n8192.md)"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--precision", default="fp16x3")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-side-by-side", action="store_true")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving session")
    ap.add_argument("--no-batch", action="store_true", help="skip the block-diagonal batch session")
    ap.add_argument("--only-batch", action="store_true", help="run only the block-diagonal batch session")
    ap.add_argument("--only-configs", action="store_true", help="run only the n=1024 and n=16384 sessions")
    ap.add_argument("--only-serve", action="store_true", help="run only the serving sessions")
    ap.add_argument("--profile-case", nargs=2, metavar=("KIND", "SIZE"),
                    help="small fixed workloads for ncu captures: 'single N' (two auto-scaled fp16x3 projections of "
                         "one n=N Gaussian matrix) or 'batch COUNT' (two projections of a COUNT-block batch)")
    ap.add_argument("--no-configs", action="store_true", help="skip the n=1024 and n=16384 sessions")
    ap.add_argument("--batch-count", type=int, default=4096)
    ap.add_argument("--serve-seconds", type=float, default=2.0)
    ap.add_argument("--workload", choices=["spectrum", "gaussian"], default="spectrum",
                    help="spectrum: Q diag(lambda) Q^T (the n=8192 configuration); gaussian: (G+G^T)/2 scaled to "
                         "norm ~1, no QR (used for profiling runs, where ncu cannot load torch's linalg library)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# distributed plumbing (replicas)
# ---------------------------------------------------------------------------

def dist_setup():
    """Rank and world size from the torchrun environment; one process per GPU
    over NCCL (gloo on a host without GPUs, where only the plumbing runs)."""
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    cuda = torch.cuda.is_available()
    if cuda:
        torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        if cuda:
            dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        else:
            dist.init_process_group("gloo")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    """The largest x over the ranks (every rank gets it)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, ms_max: float, world: int) -> float:
    """Units of all ranks per second over the slowest rank's time: each of the
    `world` replicas processed `units_per_rank` units in at most ms_max ms."""
    return world * units_per_rank / (ms_max / 1e3)


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------

def make_workload(n: int, seed: int = 0, kind: str = "spectrum"):
    """X (FP64 device, FP32-representable values) and its exact projection
    (None for the gaussian profiling workload)."""
    import torch

    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    if kind == "gaussian":
        G = torch.randn((n, n), generator=g, dtype=torch.float64, device="cuda")
        X = (0.5 / (n ** 0.5)) * (G + G.T)
        torch.cuda.synchronize()
        return X.float().double().contiguous(), None, 0.5
    G = torch.randn((n, n), generator=g, dtype=torch.float64, device="cuda")
    Q, _ = torch.linalg.qr(G)
    del G
    g.manual_seed(seed + 1)
    lam = torch.rand(n, generator=g, dtype=torch.float64, device="cuda") * 2.0 - 1.0
    A = (Q * lam) @ Q.T
    A = 0.5 * (A + A.T)
    X = A.float().double()                       # "stored in FP32"
    del A
    P = (Q * lam.clamp(min=0.0)) @ Q.T
    P = 0.5 * (P + P.T)
    del Q
    torch.cuda.synchronize()
    return X.contiguous(), P.contiguous(), float((lam < 0).double().mean())


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-f", self.path], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        if self.path and os.path.exists(self.path):
            for line in Path(self.path).read_text().splitlines():
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 8:
                    rows.append(parts)
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}

        def num(s):
            try:
                return float(s)
            except ValueError:
                return None

        sm = [num(r[0]) for r in rows if num(r[0]) is not None]
        smax = [num(r[1]) for r in rows if num(r[1]) is not None]
        loaded = [v for v in sm if smax and v >= 0.5 * max(smax)] or sm
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, val in zip(names, r[4:8]):
                if val.lower() == "active":
                    reasons.add(name)
        power = [num(r[2]) for r in rows if num(r[2]) is not None]
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "power_w_max": max(power) if power else None, "samples": len(rows)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"bf16_tflops": d.get("bf16_tflops"), "bf16_tflops_sustained": d.get("bf16_tflops_sustained"),
                "hbm_gbs": d.get("hbm_gbs"), "source": "measured"}
    return {"bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "hbm_gbs": 6800.0, "source": "fallback"}


def dense_equiv_flops(n: int, steps: int) -> float:
    """(3K + 1) 2 n^3: the reference's GEMM chain as full GEMMs."""
    return (3 * steps + 1) * 2.0 * float(n) ** 3


# ---------------------------------------------------------------------------
# serving: 64 ADMM-like streams through the library's request loop
# ---------------------------------------------------------------------------

def serve_session(offered_rate: float, seconds: float, sizes=(64, 256, 1024, 4096), n_streams: int = 64,
                  seed: int = 0, max_slots: int = 16, check_error: bool = False, admission: str = "fifo",
                  priority_n: int = 0, reserve_sms: int = 0, reserve_slots: int = 0) -> dict:
    """Closed-loop ADMM streams: stream k (n = sizes[k % 4]) waits an
    exponential think time (mean n_streams / offered_rate), perturbs its
    matrix by 1e-2 (E + E^T)/2, submits it, and waits for the projection
    before its next think time.  Returns throughput and latency percentiles."""
    import heapq

    import numpy as np
    import torch

    import psd_projection_gb300 as psd
    from psd_projection_gb300.serve import Server

    rng = np.random.default_rng(seed)
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    mats, outs, ns = [], [], []
    for k in range(n_streams):
        n = sizes[k % len(sizes)]
        G = torch.randn((n, n), generator=g, dtype=torch.float64, device="cuda")
        mats.append((0.5 / n ** 0.5) * (G + G.T))
        outs.append(torch.empty((n, n), dtype=torch.float64, device="cuda"))
        ns.append(n)
    torch.cuda.synchronize()
    mean_think = n_streams / offered_rate
    lat, lat_by_n, gpu_ms = [], {n: [] for n in sizes}, []
    with Server(hbm_budget_bytes=64 << 30, max_slots=max_slots, warm_max_iter=10, admission=admission,
                priority_n=priority_n, reserve_sms=reserve_sms, reserve_slots=reserve_slots) as srv:
        # warm the per-(slot, n) graphs outside the measured window
        for k in range(min(n_streams, 2 * len(sizes))):
            srv.submit(k, mats[k], outs[k])
        srv.drain()
        t0 = psd.serve.clock()
        t_end = t0 + seconds
        ready = [(t0 + rng.exponential(mean_think), k) for k in range(n_streams)]
        heapq.heapify(ready)
        outstanding = 0
        submitted = completed = 0
        while True:
            now = psd.serve.clock()
            while ready and ready[0][0] <= now and ready[0][0] < t_end:
                _, k = heapq.heappop(ready)
                n = ns[k]
                E = torch.randn((n, n), generator=g, dtype=torch.float64, device="cuda")
                mats[k].add_(E + E.T, alpha=0.5e-2)
                torch.cuda.current_stream().synchronize()
                srv.submit(k, mats[k], outs[k])
                outstanding += 1
                submitted += 1
            if not ready and outstanding == 0:
                break
            if ready and ready[0][0] >= t_end and outstanding == 0:
                break
            for c in srv.poll(wait=False):
                outstanding -= 1
                completed += 1
                dt = c.end_s - c.submit_s
                lat.append(dt)
                lat_by_n[c.n].append(dt)
                gpu_ms.append(c.gpu_ms)
                if c.end_s < t_end:
                    heapq.heappush(ready, (c.end_s + rng.exponential(mean_think), c.key))
            if outstanding and (not ready or ready[0][0] > psd.serve.clock()):
                time.sleep(0.0001)
        wall = psd.serve.clock() - t0
        err = None
        if check_error:
            errs = {}
            for k in range(len(sizes)):  # one stream per size: its last projection against FP64 EVD
                ref = mats[k].clone()
                psd.eig_FP64_psd(ref)
                errs[ns[k]] = psd.rel_frobenius(outs[k], ref)
            err = errs
    a = np.array(lat) * 1e3
    return {"offered_req_s": offered_rate, "admission": admission, "priority_n": priority_n,
            "reserve_sms": reserve_sms, "reserve_slots": reserve_slots, "max_slots": max_slots,
            "throughput_req_s": completed / wall,
            "completed": completed,
            "p50_ms": float(np.percentile(a, 50)) if len(a) else None,
            "p99_ms": float(np.percentile(a, 99)) if len(a) else None,
            "p50_ms_by_n": {str(n): float(np.percentile(np.array(v) * 1e3, 50)) for n, v in lat_by_n.items() if v},
            "p99_ms_by_n": {str(n): float(np.percentile(np.array(v) * 1e3, 99)) for n, v in lat_by_n.items() if v},
            "rel_frobenius_err_by_n": err, "wall_s": wall}


# ---------------------------------------------------------------------------
# config 1 (n = 1024 Gaussian) and config 3 (n = 16384 precision stress)
# ---------------------------------------------------------------------------

def config1_session(n: int = 1024, seed: int = 0) -> dict:
    """A = (G + G^T)/2, G ~ N(0,1) (seeded), stored FP32: composite_FP32 with
    a 30-step Lanczos bound on the GPU against the FP64 LAPACK dsyevd
    projection on the host; the relative Frobenius error between the two."""
    import numpy as np
    import torch

    import psd_projection_gb300 as psd
    from oracle import reference_port as rp

    g = np.random.default_rng(seed).standard_normal((n, n))
    x = (0.5 * (g + g.T)).astype(np.float32).astype(np.float64)
    t0 = time.perf_counter()
    proj, _ = rp.eig_psd(x)
    cpu_s = time.perf_counter() - t0
    d = torch.from_numpy(np.ascontiguousarray(x.T)).cuda()
    work = d.clone()
    psd.composite(work, max_iter=30)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 10
    bufs = [d.clone() for _ in range(reps)]
    e0.record()
    for b in bufs:
        psd.composite(b, max_iter=30)
    e1.record()
    torch.cuda.synchronize()
    out = bufs[-1].cpu().numpy().T
    return {"workload": "n=1024, A=(G+G^T)/2, G~N(0,1) seed 0, FP32 storage; composite_FP32 (fp16x3) with "
                        "30 Lanczos steps vs host FP64 dsyevd projection",
            "rel_frobenius_err": rp.rel_frobenius(out, proj), "gpu_ms": e0.elapsed_time(e1) / reps,
            "cpu_dsyevd_s": cpu_s, "cpu_cores": os.cpu_count()}


def config3_session(n: int = 16384, seed: int = 3) -> dict:
    """Precision stress: Q diag(lambda) Q^T, Q from the QR of a seeded
    Gaussian; 10% of lambda in |lambda| < 1e-3, 60% uniform in [-1, -1e-3],
    30% uniform in [1e-3, 10]; stored FP32.  Each mode's error against the
    exact projection Q diag(max(lambda, 0)) Q^T and its time."""
    import torch

    import psd_projection_gb300 as psd

    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    t_setup = time.perf_counter()
    G = torch.randn((n, n), generator=g, dtype=torch.float64, device="cuda")
    Q, _ = torch.linalg.qr(G)
    del G
    k1, k2 = n // 10, n // 10 + (6 * n) // 10
    u = torch.rand(n, generator=g, dtype=torch.float64, device="cuda")
    lam = torch.empty(n, dtype=torch.float64, device="cuda")
    lam[:k1] = (u[:k1] * 2.0 - 1.0) * 1e-3
    lam[k1:k2] = -1e-3 - u[k1:k2] * (1.0 - 1e-3)
    lam[k2:] = 1e-3 + u[k2:] * (10.0 - 1e-3)
    A = (Q * lam) @ Q.T
    X = (0.5 * (A + A.T)).float().double()
    del A
    P = (Q * lam.clamp(min=0.0)) @ Q.T
    P = 0.5 * (P + P.T)
    del Q
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t_setup
    runs = {}

    def timed(name, fn):
        t = X.clone()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn(t)
        e1.record()
        torch.cuda.synchronize()
        runs[name] = {"ms": e0.elapsed_time(e1), "rel_frobenius_err": psd.rel_frobenius(t, P)}
        del t

    P16, P32 = psd.SCHEDULE_FP16, psd.SCHEDULE_FP32
    timed("plain_fp32_simt", lambda t: psd.composite(t, psd.PRECISIONS["fp32_simt"], P32))
    timed("fp16x3", lambda t: psd.composite(t, psd.PRECISIONS["fp16x3"], P32))
    timed("bf16x9", lambda t: psd.composite(t, psd.PRECISIONS["bf16x9"], P32))
    timed("bf16_bulk_only", lambda t: psd.composite(t, psd.PRECISIONS["bf16"], P16))
    timed("fp16_bulk_only", lambda t: psd.composite(t, psd.PRECISIONS["fp16"], P16))
    timed("fp8_bulk_only", lambda t: psd.composite(t, psd.PREC_FP8, psd.SCHEDULE_FP8))
    for r in (1, 2):
        timed(f"bf16_bulk+{r}x_bf16x9_refine", lambda t, r=r: psd.composite_mixed(t, "bf16", "bf16x9", r))
        timed(f"fp16_bulk+{r}x_fp16x3_refine", lambda t, r=r: psd.composite_mixed(t, "fp16", "fp16x3", r))
        timed(f"fp8_bulk+{r}x_fp16x3_refine", lambda t, r=r: psd.composite_mixed(t, "fp8", "fp16x3", r))
    return {"workload": f"n={n} precision stress: 10% |lambda|<1e-3, 60% U[-1,-1e-3], 30% U[1e-3,10], "
                        "Q=QR(N(0,1)) seed 3, FP32 storage; bulk = one-term products (FP16 / BF16 on the FP16 "
                        "schedule, FP8 E4M3 on the FP8 schedule: the FP16 table with safety factor 1.5), "
                        "refinement = the FP32 table's final quintic in split precision",
            "setup_s": setup_s, "runs": runs,
            "note": "FP8 products: tcgen05.mma kind::f8f6f4 on 128x128 tiles, E4M3 operand copies beside the "
                    "FP16 pair the refinement reads"}


# ---------------------------------------------------------------------------
# block-diagonal batch: 4096 uneven blocks
# ---------------------------------------------------------------------------

def deflation_session(n: int = 1024, seed: int = 1) -> dict:
    """The eigenpair / deflation routines (the reference's work-in-progress
    family) at n = 1024 on the uniform spectrum lambda in [-10, 10] (the
    reference tests' construction): GPU wall time of one call (after a warm
    call), error against the host FP64 EVD projection, and the CPU
    restatement's time on the same input where it finishes in seconds."""
    import numpy as np
    import torch

    import psd_projection_gb300 as psd
    from oracle import deflation_port as dp
    from oracle import reference_port as rp

    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.random((n, n)) - 0.5)
    x = (q * np.linspace(-10.0, 10.0, n)) @ q.T
    proj, _ = rp.eig_psd(x)
    d = torch.from_numpy(np.ascontiguousarray(x)).cuda()

    def gpu(fn, reps=3):
        w = d.clone()
        fn(w)
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(reps):
            w = d.clone()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn(w)
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        return best * 1e3, w.cpu().numpy()

    def cpu(fn):
        t0 = time.perf_counter()
        out = fn()
        return time.perf_counter() - t0, out

    res = {}
    ms, out = gpu(lambda w: psd.composite_FP32_auto_scale_deflate(w, k=40, ortho_tol=1e-8))
    cs, cout = cpu(lambda: dp.composite_auto_scale_deflate(x, "fp32", k=40, ortho_tol=1e-8))
    res["composite_FP32_auto_scale_deflate_k40"] = {
        "gpu_ms": ms, "rel_frobenius_err": rp.rel_frobenius(out, proj), "cpu_port_s": cs,
        "cpu_port_err": rp.rel_frobenius(cout, proj), "note": "ortho_tol 1e-8; 1024 Lanczos steps"}
    ms, out = gpu(lambda w: psd.eig_FP64_deflate(w, k=40))
    res["eig_FP64_deflate_k40"] = {"gpu_ms": ms, "rel_frobenius_err": rp.rel_frobenius(out, proj)}
    ms, out = gpu(lambda w: psd.composite_FP16_auto_scale_deflate(w, k=100))
    res["composite_FP16_auto_scale_deflate_k100"] = {"gpu_ms": ms, "rel_frobenius_err": rp.rel_frobenius(out, proj)}
    ms, _ = gpu(lambda w: psd.compute_eigenpairs(w, 40, ortho_tol=1e-8))
    res["compute_eigenpairs_k40"] = {"gpu_ms": ms}
    rr = np.random.default_rng(7).random((1000, 1000))
    a = torch.from_numpy(rr + rr.T).cuda()
    psd.lobpcg(a, 100)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lr = psd.lobpcg(a, 100)
    torch.cuda.synchronize()
    lms = (time.perf_counter() - t0) * 1e3
    w = np.linalg.eigvalsh(rr + rr.T)[::-1][:100]
    res["lobpcg_n1000_m100"] = {"gpu_ms": lms, "iters": lr["iters"],
                                "max_eig_err": float(np.abs(lr["D"].cpu().numpy() - w).max())}
    res["workload"] = (f"n={n}, A = Q diag(linspace(-10, 10)) Q^T, Q = QR(U[-0.5, 0.5]) seed {seed}; "
                       "lobpcg on R + R^T, R ~ U[0, 1], n = 1000, m = 100 (the reference's LOBPCG.Random)")
    return res


def batched_session(count: int = 4096, seed: int = 0, replays: int = 5, evd_sample: int = 8) -> dict:
    """4096 blocks, n log-uniform in [16, 512] (seeded), entries (G + G^T)/2,
    stored FP32; the whole batch projected by one plan as one CUDA graph (the
    plan's own, psdgb_batch_project_graph, and one the caller captures with
    torch), against the same blocks projected one call at a time."""
    import numpy as np
    import torch

    import psd_projection_gb300 as psd
    from oracle import reference_port as rp
    from psd_projection_gb300.batch import BatchPlan

    rng = np.random.default_rng(seed)
    sizes = [int(round(v)) for v in np.exp(rng.uniform(np.log(16), np.log(512), count))]
    offs = np.concatenate([[0], np.cumsum([n * n for n in sizes])])
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    pristine = torch.empty(int(offs[-1]), dtype=torch.float64, device="cuda")
    for b, n in enumerate(sizes):
        G = torch.randn((n, n), generator=g, dtype=torch.float64, device="cuda")
        pristine[offs[b]:offs[b + 1]].copy_((0.5 * (G + G.T)).float().double().reshape(-1))
    torch.cuda.synchronize()
    plan = BatchPlan(sizes)
    scratch = pristine.clone()
    best = plan.autotune(scratch)
    info = plan.info()
    tuned = plan.tuning()
    # the alternatives the autotuner chose between, direct launches: the route of
    # the blocks of n <= 128 (on chip / per-product launches) and the tile shape
    # of the larger ones (256 x 256 pair tiles / 128 x 128 tiles only)
    routes = {}
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(**cfg):
        plan.configure(**cfg)
        plan.project(scratch)
        ev0.record()
        for _ in range(3):
            plan.project(scratch)
        ev1.record()
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / 3

    if tuned["small_blocks"] > 0:
        for chip in (1, 0):
            routes["ms_small_on_chip" if chip else "ms_small_per_product"] = timed(small_on_chip=chip)
        plan.configure(small_on_chip=tuned["small_on_chip"])
    if tuned["num_pair_tiles"] > 0:
        for pairs in (1, 0):
            routes["ms_pair_tiles" if pairs else "ms_single_tiles_only"] = timed(pair_tiles=pairs)
        plan.configure(pair_tiles=tuned["pair_tiles"])
    work = pristine.clone()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        plan.project(scratch, stream=side)
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        work.copy_(pristine)
        plan.project(work)
    graph.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(replays):
        graph.replay()
    e1.record()
    torch.cuda.synchronize()
    ms_batch = e0.elapsed_time(e1) / replays
    # the plan's own graph (stream priorities kept), the same input copy before each launch
    work.copy_(pristine)
    plan.project_graph(work)  # captures (for this pointer) and runs once
    e0.record()
    for _ in range(replays):
        work.copy_(pristine)
        plan.project_graph(work)
    e1.record()
    torch.cuda.synchronize()
    ms_plan_graph = e0.elapsed_time(e1) / replays
    # copy-only cost inside the graph, for reference
    e0.record()
    for _ in range(replays):
        scratch.copy_(pristine)
    e1.record()
    torch.cuda.synchronize()
    ms_copy = e0.elapsed_time(e1) / replays
    # one call at a time (the reference's usage: one projection per block)
    one = pristine.clone()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for b, n in enumerate(sizes):
        psd.composite(one[offs[b]:offs[b + 1]].view(n, n))
    torch.cuda.synchronize()
    ms_one = (time.perf_counter() - t0) * 1e3
    diffs = []
    for b, n in enumerate(sizes):
        a = work[offs[b]:offs[b + 1]]
        c = one[offs[b]:offs[b + 1]]
        diffs.append(float(torch.linalg.vector_norm(a - c) / torch.linalg.vector_norm(c)))
    evd = {}
    for b in sorted(range(count), key=lambda i: -sizes[i])[:evd_sample // 2] + list(range(evd_sample // 2)):
        n = sizes[b]
        x = pristine[offs[b]:offs[b + 1]].cpu().numpy().reshape(n, n).T
        proj, _ = rp.eig_psd(x)
        y = work[offs[b]:offs[b + 1]].cpu().numpy().reshape(n, n).T
        evd[str(n)] = rp.rel_frobenius(y, proj)
    plan.close()
    dense = sum(62.0 * n ** 3 for n in sizes)
    return {"blocks": count, "sizes": "log-uniform [16, 512], seed 0", "sum_n3": float(sum(n ** 3 for n in sizes)),
            "ms_per_batch_graph": ms_batch, "ms_per_batch_plan_graph": ms_plan_graph,
            "ms_input_copy_in_graph": ms_copy, "ms_one_call_at_a_time": ms_one,
            "speedup_vs_one_call_at_a_time": ms_one / ms_plan_graph, "batches_per_s": 1e3 / ms_plan_graph,
            "dense_equiv_tflops": dense / (ms_plan_graph / 1e3) / 1e12,
            "figures_from": "ms_per_batch_plan_graph (psdgb_batch_project_graph; the input copy included)",
            "max_rel_diff_vs_one_call": max(diffs), "rel_frobenius_err_vs_evd_sample": evd,
            "autotune": {"best_ms": best, "acc_mode": info["acc_mode"], "tile_order": info["tile_order"],
                         "small_on_chip": tuned["small_on_chip"], "small_blocks": tuned["small_blocks"],
                         "pair_tiles": tuned["pair_tiles"], "num_pair_tiles": tuned["num_pair_tiles"],
                         "serpentine": tuned["serpentine"],
                         "num_tiles": info["num_tiles"], "device_bytes": info["device_bytes"], **routes}}


# ---------------------------------------------------------------------------
# CPU baseline: FP64 LAPACK dsyevd projection (eig_FP64_psd's math)
# ---------------------------------------------------------------------------

def cpu_model() -> str:
    """The host CPU's model name (lscpu), for the baseline records."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        fields = dict(line.split(":", 1) for line in out.splitlines() if ":" in line)
        name = fields.get("Model name", "").strip()
        vendor = fields.get("Vendor ID", "").strip()
        return " ".join(x for x in (vendor, name) if x) or "unknown"
    except (OSError, subprocess.SubprocessError, ValueError):
        return "unknown"


def cpu_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_evd_projection_time(xs) -> float:
    """Seconds for one FP64 LAPACK dsyevd projection V max(L, 0) V^T of the
    full host matrix xs (scipy eigh 'evd', all host cores)."""
    from oracle import reference_port as rp

    t0 = time.perf_counter()
    rp.eig_psd(xs)
    return time.perf_counter() - t0


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------

def lib_check_error(psd) -> bool:
    """True when a bounded device-side wait gave up during asynchronous work."""
    return psd._capi.lib().psdgb_check_device_error() != 0


def profile_case(kind: str, size: str) -> None:
    """Fixed small workloads to run under ncu (no timing, no oracle)."""
    import numpy as np
    import torch

    import psd_projection_gb300 as psd

    n = int(size)
    if kind == "single":
        g = torch.Generator(device="cuda")
        g.manual_seed(0)
        G = torch.randn((n, n), generator=g, dtype=torch.float64, device="cuda")
        X = ((0.5 / n ** 0.5) * (G + G.T)).float().double().contiguous()
        del G
        for _ in range(2):
            psd.composite(X.clone())
    elif kind == "batch":
        from psd_projection_gb300.batch import BatchPlan

        rng = np.random.default_rng(0)
        sizes = [int(round(v)) for v in np.exp(rng.uniform(np.log(16), np.log(512), n))]
        offs = np.concatenate([[0], np.cumsum([m * m for m in sizes])])
        g = torch.Generator(device="cuda")
        g.manual_seed(0)
        d = torch.empty(int(offs[-1]), dtype=torch.float64, device="cuda")
        for b, m in enumerate(sizes):
            G = torch.randn((m, m), generator=g, dtype=torch.float64, device="cuda")
            d[offs[b]:offs[b + 1]].copy_((0.5 * (G + G.T)).float().double().reshape(-1))
        plan = BatchPlan(sizes)
        for _ in range(2):
            plan.project(d.clone())
    else:
        raise SystemExit("--profile-case KIND is 'single' or 'batch'")
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": kind, "size": n}))


def serving_sessions(args) -> dict:
    sessions = [serve_session(r, args.serve_seconds, check_error=(r == 2000.0)) for r in (250.0, 500.0, 2000.0)]
    sessions += [serve_session(r, args.serve_seconds, admission="shortest_first") for r in (500.0, 2000.0)]
    # Small requests (n <= 1024) first: high-priority streams, 16 SMs kept free of the n = 4096 products,
    # and 8 of 24 slots kept for them.
    sessions += [serve_session(2000.0, args.serve_seconds, admission=a, max_slots=24, priority_n=1024,
                               reserve_sms=16, reserve_slots=8) for a in ("fifo", "shortest_first")]
    return {"workload": "64 closed-loop ADMM-like streams, n uniform over {64,256,1024,4096} (16 streams each), "
                        "next matrix = previous + 1e-2 (E+E^T)/2, exponential think time for the offered rate; "
                        "fp16x3, warm-started Lanczos (10 steps), 16 slots, CUDA-graph replay",
            "sessions": sessions}


def run_ours(args, rank, world):
    import torch

    import psd_projection_gb300 as psd

    n, K, W = args.n, args.steps, args.warmup
    prec = psd.PRECISIONS[args.precision]
    sched = psd.SCHEDULE_FP16 if args.precision == "fp16" else psd.SCHEDULE_FP32
    X, P, neg_frac = make_workload(n, seed=0, kind=args.workload)
    # One resident input per step: every step reads a fresh 537 MB matrix (> L2).
    inputs = [torch.empty_like(X) for _ in range(W + K)]
    stream = torch.cuda.current_stream()

    def refill():
        for t in inputs:
            t.copy_(X)
        torch.cuda.synchronize()

    refill()
    # The timed steps run through the asynchronous entry point: the host
    # enqueues every step's projection ahead of the GPU (one workspace on one
    # stream), so the GPU never waits for the host to launch the next step.
    ws, lz = psd.async_buffers(n, prec)
    for i in range(W):
        psd.composite_async(inputs[i], ws, lz, prec, sched, stream=stream)
    torch.cuda.synchronize()
    if lib_check_error(psd):
        raise RuntimeError("device error in the warm-up steps")

    lib = psd._capi.lib()
    lib.psdgb_product_timing_read(None, None, None, 1)
    lib.psdgb_product_timing_enable(1)
    launches0 = psd.kernel_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        barrier(world)
        torch.cuda.synchronize()
        e0.record(stream)
        for i in range(K):
            psd.composite_async(inputs[W + i], ws, lz, prec, sched, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
    if lib_check_error(psd):
        raise RuntimeError("device error in the timed steps")
    lib.psdgb_product_timing_enable(0)
    launches = psd.kernel_launch_count() - launches0
    ms_total = e0.elapsed_time(e1)
    ms_total = max_over_ranks(ms_total, world)
    import ctypes

    pms, pl, pfl = ctypes.c_double(), ctypes.c_uint64(), ctypes.c_double()
    lib.psdgb_product_timing_read(ctypes.byref(pms), ctypes.byref(pl), ctypes.byref(pfl), 1)
    err = psd.rel_frobenius(inputs[W + K - 1], P) if P is not None else None
    clocks = clk.summary()

    value = whole_job_rate(K, ms_total, world)
    steps_filter = 7 if sched == psd.SCHEDULE_FP16 else 10
    tc = {
        "dense_equiv_tflops": value / world * dense_equiv_flops(n, steps_filter) / 1e12,
        "executed_mma_tflops": (pfl.value / max(pl.value, 1)) / (pms.value / max(pl.value, 1) / 1e3) / 1e12
        if pl.value else None,
    }
    peaks = measured_peaks()
    per_launch_flops = pfl.value / max(pl.value, 1)
    per_launch_ms = pms.value / max(pl.value, 1)
    achieved = per_launch_flops / (per_launch_ms / 1e3) / 1e12 if pl.value else None
    # Each product launch lasts about a millisecond and is timed alone by its
    # own events: the burst peak is its denominator.
    peak = peaks["bf16_tflops"]
    np_ = -(-n // 128) * 128
    wide = args.precision in ("fp16", "bf16", "fp16x3", "bf16x3") and np_ >= 2048
    kernel = (f"tc_pairwide_kernel (256x256 tiles on CTA pairs, tcgen05.mma.cta_group::2, {args.precision} split "
              "operands, K chunks summed in FP32 registers)"
              if wide else f"tc_group_kernel (128x128 tiles, {args.precision} split operands)")
    roofline = {
        "bound": "tensor", "kernel": kernel,
        "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
        "frac": (achieved / peak) if achieved else None,
        "peak_source": f"{peaks['source']} bf16_tflops (burst; of {peaks['source']})",
        "frac_of_sustained": (achieved / peaks["bf16_tflops_sustained"])
        if achieved and peaks.get("bf16_tflops_sustained") else None,
        "flops_per_launch": per_launch_flops, "ms_per_launch": per_launch_ms, "launches": pl.value,
        "flops_counted": "MMA flops of the lower-triangle 128x128 tiles: term products x 2 x 128 x 128 x K "
                         "per tile (K doubled for the final dual product); the 1.5 % of above-diagonal work the "
                         "256x256 tiles also do is not counted",
        "share_of_step": (pms.value / ms_total) if ms_total else None,
        "traffic": TRAFFIC_PER_LAUNCH.get((n, args.precision, wide)),
        "traffic_source": TRAFFIC_SOURCE if (n, args.precision, wide) in TRAFFIC_PER_LAUNCH else None,
    }

    out = {
        "metric": METRIC, "value": value, "unit": "proj/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms_total / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": args.precision, "data": "synthetic: A = Q diag(lambda) Q^T, Q = QR(N(0,1)) seed 0, "
                                          "lambda ~ U[-1,1] seed 1, stored FP32, passed as FP64",
        "config": {"workload": f"single dense projection n={n} (lambda uniform in [-1,1]), "
                               "composite_FP32_auto_scale", "n": n, "precision": args.precision,
                   "lanczos_steps": 20, "filter_steps": steps_filter,
                   "l2": "each step projects its own resident input (8n^2 B > L2); no flush",
                   "negative_fraction": neg_frac, "rel_frobenius_err": err, "replicas": world},
        "tc_tflops": tc, "gpu_launches": launches, "clocks": clocks, "roofline": roofline,
    }
    if rank != 0 or P is None:
        return out

    # e2e: the C-ABI host-buffer calls, both copies of every step inside the
    # timed region.  psdgb_project_host_many projects the K steps' host
    # matrices in one call (copies of neighbouring steps overlap each
    # projection); each step reads its input from pinned host memory and
    # writes its result back (two input and two output buffers in rotation).
    Xh = [torch.empty((n, n), dtype=torch.float64, pin_memory=True) for _ in range(2)]
    for h in Xh:
        h.copy_(X.cpu())
    Oh = [torch.empty((n, n), dtype=torch.float64, pin_memory=True) for _ in range(2)]
    Ke = max(3, K)
    psd.project_host_many("composite_FP32", Xh, Oh)  # warm
    t0 = time.perf_counter()
    psd.project_host_many("composite_FP32", [Xh[i % 2] for i in range(Ke)], [Oh[i % 2] for i in range(Ke)])
    te = time.perf_counter() - t0
    e2e_err = psd.rel_frobenius(Oh[(Ke - 1) % 2].cuda(), P)
    # The same through one synchronous call per matrix (no overlap).
    Ks = max(2, min(K, 5))
    t0 = time.perf_counter()
    for _ in range(Ks):
        psd.project_host("composite_FP32", Xh[0], Oh[0])
    ts = time.perf_counter() - t0
    out["e2e"] = {"value": Ke / te, "unit": "proj/s", "h2d_bytes_per_step": 8 * n * n,
                  "d2h_bytes_per_step": 8 * n * n, "steps": Ke,
                  "api": "psdgb_project_host_many(\"composite_FP32\") over the steps' pinned host matrices",
                  "rel_frobenius_err": e2e_err,
                  "one_call_per_matrix": {"value": Ks / ts, "unit": "proj/s",
                                          "api": "psdgb_project_host(\"composite_FP32\")"}}

    if not args.no_side_by_side:
        side = {}
        for name, steps in (("fp16", 3), ("bf16x9", 3), ("bf16x6", 3), ("bf16x3", 3), ("fp32_simt", 1)):
            p = psd.PRECISIONS[name]
            s = psd.SCHEDULE_FP16 if name == "fp16" else psd.SCHEDULE_FP32
            t = inputs[0]
            t.copy_(X)
            psd.composite(t, p, s, auto_scale=True)
            for j in range(steps):
                inputs[1 + j].copy_(X)
            torch.cuda.synchronize()
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record()
            for j in range(steps):
                psd.composite(inputs[1 + j], p, s, auto_scale=True)
            ev1.record()
            torch.cuda.synchronize()
            ms = ev0.elapsed_time(ev1) / steps
            side[name] = {"proj_s": 1e3 / ms, "ms": ms, "rel_frobenius_err": psd.rel_frobenius(inputs[steps], P),
                          "method": {"fp16": "composite_FP16", "bf16x9": "composite_FP32_emulated",
                                     "fp32_simt": "plain FP32 (CUDA cores)"}.get(name, name)}
        # FP32 in / FP32 out (psdgb_composite_auto_scale_f32, asynchronous):
        # the same projection for callers whose iterate is FP32.
        x32 = [X.float() for _ in range(4)]
        psd.composite_f32(x32[0])
        torch.cuda.synchronize()
        for t32 in x32[1:]:
            t32.copy_(X)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for t32 in x32[1:]:
            psd.composite_f32(t32)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 3
        side["fp16x3_fp32_io"] = {"proj_s": 1e3 / ms, "ms": ms,
                                  "rel_frobenius_err": psd.rel_frobenius(x32[-1].double(), P),
                                  "method": "psdgb_composite_auto_scale_f32 (FP32 input and output)"}
        out["side_by_side"] = side

    if not args.no_batch:
        out["batched"] = batched_session(count=args.batch_count)

    if not args.no_configs:
        out["config1"] = config1_session()
        out["config3"] = config3_session()
        out["deflation"] = deflation_session()

    if not args.no_serve:
        out["serving"] = serving_sessions(args)

    if world == 1 and not args.no_cpu_baseline:
        xs = X.cpu().numpy()
        t = cpu_evd_projection_time(xs)
        out["cpu_baseline"] = {"value": 1.0 / t, "unit": "proj/s", "cores": cpu_cores(), "cpu": cpu_model(),
                               "kind": "port",
                               "sample": f"one FP64 LAPACK dsyevd projection V max(L,0) V^T (scipy eigh 'evd') of "
                                         f"the full {n}x{n} matrix, {t:.2f} s"}
    return out


def run_reference(args, rank, world):
    import torch

    if rank != 0:
        return None
    n, K, W = args.n, args.steps, args.warmup
    X, P, _ = make_workload(n, seed=0)
    xs = X.cpu().numpy()
    # CPU path: one full FP64 dsyevd projection per step, on all host cores.
    for _ in range(W):
        cpu_evd_projection_time(xs)
    t0 = time.perf_counter()
    times = [cpu_evd_projection_time(xs) for _ in range(K)]
    wall = time.perf_counter() - t0
    value = K / wall
    out = {
        "metric": METRIC, "value": value, "unit": "proj/s", "n_gpus": 1, "steps": K, "warmup": W,
        "ms_per_step": 1e3 * wall / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (same workload as the default arm)", "impl": "reference",
        "config": {"workload": f"single dense projection n={n} (lambda uniform in [-1,1])", "n": n},
        "cpu_baseline": {"value": value, "unit": "proj/s", "cores": cpu_cores(), "cpu": cpu_model(), "kind": "port",
                         "sample": f"one FP64 LAPACK dsyevd projection V max(L,0) V^T (scipy eigh 'evd') of the "
                                   f"full {n}x{n} matrix per step; {K} steps in {wall:.1f} s (min "
                                   f"{min(times):.2f} s, max {max(times):.2f} s)"},
        "e2e": {"value": value, "unit": "proj/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if not args.no_side_by_side:
        out["gpu_methods"] = reference_gpu_methods(X, P)
    return out


def reference_gpu_methods(X, P, reps: int = 2) -> dict:
    """The reference's three auto-scaled GPU methods replayed on cuBLAS /
    cuSOLVER (oracle/ref_replay.cu) on the same matrix: proj/s as shipped
    (cudaMalloc / cudaFree inside every call) and with caller workspaces, and
    the relative Frobenius error against the exact projection."""
    import torch

    from oracle import gpu_replay

    res = {}
    for method in ("composite_FP32", "composite_FP16", "composite_FP32_emulated"):
        try:
            row = {}
            ws = gpu_replay.Workspaces(method, X.shape[0])
            for mode, w in (("per_call_alloc", None), ("caller_workspace", ws)):
                t = X.clone()
                gpu_replay.auto_scale(method, t, w)  # warm (handles, kernels, allocator)
                ts = [X.clone() for _ in range(reps)]
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for t in ts:
                    gpu_replay.auto_scale(method, t, w)
                e1.record()
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1) / reps
                err = float(torch.linalg.matrix_norm(ts[-1] - P) / torch.linalg.matrix_norm(P))
                row[mode] = {"proj_s": 1e3 / ms, "ms": ms, "rel_frobenius_err": err}
                del ts
            del ws
            row["what"] = {"composite_FP32": "cublasSgemm chain (FP32, default math mode)",
                           "composite_FP16": "cublasGemmEx FP16 x FP16 -> FP32, CUBLAS_COMPUTE_32F_FAST_16F",
                           "composite_FP32_emulated": "cublasGemmEx FP32, CUBLAS_COMPUTE_32F_EMULATED_16BFX9"}[method]
            res[method + "_auto_scale"] = row
        except Exception as exc:  # noqa: BLE001 - report, do not fail the CPU arm
            res[method + "_auto_scale"] = {"unavailable": repr(exc)[:300]}
        torch.cuda.empty_cache()
    res["how"] = ("oracle/ref_replay.cu: the reference's cuBLAS / cuSOLVER call sequence (Lanczos with host reads "
                  "of every Ddot / Dnrm2, the GEMM chain, Sgeam symmetrisation, blocking conversions) on the "
                  "legacy default stream; CUDA events around `reps` calls after one warm call")
    return res


def main():
    args = parse_args()
    rank, world = dist_setup()
    if args.only_batch:
        print(json.dumps({"batched": batched_session(count=args.batch_count)}))
        return
    if args.profile_case:
        profile_case(*args.profile_case)
        return
    if args.only_serve:
        print(json.dumps({"serving": serving_sessions(args)}))
        return
    if args.only_configs:
        print(json.dumps({"config1": config1_session(), "config3": config3_session(),
                          "deflation": deflation_session()}))
        return
    res = run_reference(args, rank, world) if args.impl == "reference" else run_ours(args, rank, world)
    if rank == 0 and res is not None:
        print(json.dumps(res))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
