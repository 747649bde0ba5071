"""Shared helpers for the tests: fixtures, error metrics, seeded cases."""
from __future__ import annotations

import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# Tolerances (per node and component, relative to the FP64 sum of the
# absolute contributions |d_c| (r^-14 + r^-8/2) of the node's edges):
TOL_VS_REFERENCE = 1e-5   # GPU vs the reference's CPU result (FP32 reordering)
TOL_NORMWISE_F64 = 1e-6   # GPU vs FP64 oracle: max|df| / max|f|
TOL_PERNODE_F64 = 4e-6    # GPU vs FP64 oracle per node (FP32 per-edge arithmetic)


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name: str) -> dict:
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def oracle_param(O, case: dict):
    if str(case["map"]) == "moldyn":
        return O.lj_param(float(case["cutoff"]) ** 2, float(case["side"]), True)
    return O.lj_param(float(case["param"][0]), 0.0, False)


def map_idx_of(case: dict) -> int:
    return 0 if str(case["map"]) == "moldyn" else 1


def scaled_error(f, g, sabs):
    """max over nodes/components of |f - g| / sabs (nodes with sabs == 0 must match exactly)."""
    f = np.asarray(f, np.float64)
    g = np.asarray(g, np.float64)
    d = np.abs(f - g)
    zero = sabs == 0
    if np.any(d[zero] != 0):
        return np.inf
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(zero, 0.0, d / np.where(zero, 1.0, sabs))
    return float(r.max()) if r.size else 0.0


def normwise_error(f, f64):
    f64 = np.asarray(f64, np.float64)
    m = np.abs(f64).max() if f64.size else 0.0
    if m == 0:
        return float(np.abs(np.asarray(f, np.float64)).max()) if f64.size else 0.0
    return float(np.abs(np.asarray(f, np.float64) - f64).max() / m)


def random_box(n: int, rho: float, seed: int):
    rng = np.random.Generator(np.random.PCG64(seed))
    L = np.float32((n / rho) ** (1.0 / 3.0))
    pos = (rng.random((n, 3), dtype=np.float32) * L).astype(np.float32)
    pos[pos >= L] = 0.0
    return pos, L
