"""Generate the golden fixtures under tests/golden/.

  kat.json             the reference's own known-answer tests for this path,
                       transcribed from its test sources (file:line cited in
                       each entry)
  rng.json             the first values of the seeded Lanczos start vector
                       (pins the SplitMix64 stream shared by the CUDA path and
                       the oracle)
  coefficients.json    the FP32 per-step filter coefficients after the safety
                       scaling, as the reference computes them
  cases.npz            seeded small inputs with the oracle's projections
                       (FP64 EVD and the FP32 composite restatement)
  reference_symbols.txt  C++ symbols the reference library exports for the
                       path's entry points (from oracle/_ref, built by
                       oracle/build_ref.sh when the reference sources exist)

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle import reference_port as rp  # noqa: E402

# Entry points on the path (include/psd_projection/*.h of the reference).
PATH_FUNCTIONS = ("composite_FP16", "composite_FP16_auto_scale", "composite_FP32", "composite_FP32_auto_scale",
                  "composite_FP32_emulated", "composite_FP32_emulated_auto_scale", "approximate_two_norm",
                  "eig_FP64_psd", "eig_FP32_psd")


def kat() -> dict:
    return {
        "composite_fp32_deterministic": {
            "source": "test/composite_FP32_test.hpp:18-78",
            "input_over_15": [[1.0, 2.0, 3.0], [2.0, 5.0, 6.0], [3.0, 6.0, 9.0]],
            "expected": [[0.0667, 0.1333, 0.2000], [0.1333, 0.3333, 0.4000], [0.2000, 0.4000, 0.6000]],
            "tolerance": 1e-3,
            "call": "composite_FP32 (no scaling)",
        },
        "composite_simple5": {
            "source": "test/composite_FP32_test.hpp:249-290",
            "diagonal": [1.0, -2.0, 3.0, -4.0, 5.0],
            "expected_diagonal": [1.0, 0.0, 3.0, 0.0, 5.0],
            "tolerance": 1e-3,
            "call": "auto-scaled composite (the reference calls its deflate variant; the expectation holds for "
                    "any correct projection)",
        },
        "lanczos_two_norm": {
            "source": "test/lanczos_test.hpp:8-42",
            "matrix": [[4.0, 1.0, 2.0, 0.0, 0.0], [1.0, 3.0, 0.0, 1.0, 0.0], [2.0, 0.0, 5.0, 1.0, 1.0],
                       [0.0, 1.0, 1.0, 2.0, 1.0], [0.0, 0.0, 1.0, 1.0, 3.0]],
            "two_norm": 7.0890,
            "two_norm_rounding": 5e-5,
            "max_iter": 50,
            "tol": 1e-6,
            "assert": "lo <= two_norm <= up",
            "note": "two_norm is ||A||_2 = 7.0890125506 rounded to 4 decimals; a converged lower bound exceeds "
                    "the rounded figure, so the check allows its rounding half-unit",
        },
        "oracle_bars": {
            "uniform_scaled_rel": {"source": "test/composite_FP32_test.hpp:80-129", "n": 1000, "radius": 1.0,
                                   "rel_frobenius_max": 1e-3},
            "uniform_autoscaled_abs": {"source": "test/composite_FP32_test.hpp:201-247", "n": 1024,
                                       "radius": 10.0, "abs_frobenius_max": 0.1},
            "fp16_random_rel": {"source": "test/composite_FP16_test.hpp:67-138", "n": [100, 1000],
                                "rel_frobenius_max": 1e-3},
        },
    }


def cases() -> dict:
    out = {}
    for n, seed in ((16, 1), (64, 2), (100, 3)):
        rng = np.random.default_rng(seed)
        q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        lam = rng.uniform(-1.0, 1.0, n)
        x = (q * lam) @ q.T
        x = 0.5 * (x + x.T)
        proj, _ = rp.eig_psd(x)
        out[f"x_{n}"] = x
        out[f"evd_{n}"] = proj
        out[f"fp32_{n}"] = rp.composite_fp32(x)
    return out


def reference_symbols() -> list[str] | None:
    sym = ROOT / "oracle" / "_ref" / "symbols.txt"
    if not sym.exists():
        return None
    names = [s.strip() for s in sym.read_text().split() if s.strip()]
    keep = []
    for s in names:
        for f in PATH_FUNCTIONS:
            if s.startswith(f"_Z{len(f)}{f}"):
                keep.append(s)
    return sorted(keep)


def main() -> None:
    (HERE / "kat.json").write_text(json.dumps(kat(), indent=1) + "\n")
    sv = rp.start_vector(8, rp.DEFAULT_SEED)
    (HERE / "rng.json").write_text(json.dumps({"seed": rp.DEFAULT_SEED, "first8": [float(v) for v in sv]},
                                              indent=1) + "\n")
    coeffs = {s: [[float(v) for v in t] for t in rp.schedule_coefficients(s)] for s in ("fp32", "fp16")}
    (HERE / "coefficients.json").write_text(json.dumps(coeffs, indent=1) + "\n")
    np.savez_compressed(HERE / "cases.npz", **cases())
    syms = reference_symbols()
    if syms is not None:
        (HERE / "reference_symbols.txt").write_text("\n".join(syms) + "\n")
    print("golden fixtures written to", os.path.relpath(HERE, ROOT))


if __name__ == "__main__":
    main()
