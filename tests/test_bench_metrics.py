"""bench.py's own measurement arithmetic, on the CPU: its FP64 recomputation
of the forces (the force-error fields' reference) against the oracle's FP64
reduction, the per-result error metric on known perturbations, and the
roofline traffic read from the committed ncu summary."""
import numpy as np

import bench
from helpers import load_golden, random_box


def test_fp64_forces_equal_the_oracle(oracle_lib):
    O = oracle_lib
    pos, side = random_box(4096, bench.DENSITY, 11)
    edges = O.neighbor_half_list(pos, float(side), np.float32(bench.CUTOFF * bench.CUTOFF))
    f, sabs, sinf = bench.fp64_forces(pos, edges, float(side), bench.CUTOFF)
    g, gabs = O.lj_reduce_f64(pos.astype(np.float64), edges,
                              O.lj_param(bench.CUTOFF * bench.CUTOFF, float(side), True))
    scale = np.abs(g).max()
    assert np.abs(f - g).max() <= 1e-12 * scale
    assert np.allclose(sabs, gabs, rtol=1e-12, atol=0)
    assert np.all(sinf <= sabs.sum(axis=1) * (1 + 1e-12))


def test_fp64_forces_on_a_golden_case(oracle_lib):
    O = oracle_lib
    c = load_golden("moldyn_random_2048")
    pos32 = c["pos"].astype(np.float32)
    f, _, _ = bench.fp64_forces(pos32, c["edges"], float(c["side"]), float(c["cutoff"]))
    g, _ = O.lj_reduce_f64(pos32.astype(np.float64), c["edges"],
                           O.lj_param(float(c["cutoff"]) ** 2, float(c["side"]), True))
    assert np.abs(f - g).max() <= 1e-12 * np.abs(g).max()


def test_per_result_metric():
    g = np.array([[1.0, 0.0, 0.0], [0.0, 2.0, 0.0], [1e-6, 0.0, 0.0], [0.0, 0.0, 4.0]])
    sinf = np.array([1.0, 2.0, 1.0, 4.0])
    sabs = np.ones((4, 3))
    f = g.copy()
    f[0, 0] += 1e-7       # |f| = 1: 1e-7
    f[1, 1] -= 4e-7       # |f| = 2: 2e-7
    f[2, 0] += 2**-10 * 1e-6  # |f| = 1e-6 < 2^-10 sinf = 2^-10: the floor applies
    err = bench.force_err(f, g, sabs, sinf)
    res = np.array([1e-7, 2e-7, (2**-10 * 1e-6) / 2**-10, 0.0])
    assert np.isclose(err["per_result"]["max"], res.max(), rtol=1e-9)
    assert np.isclose(err["per_result"]["p50"], np.percentile(res, 50), rtol=1e-9)
    assert np.isclose(err["normwise"], 4e-7 / 4.0, rtol=1e-9)
    assert err["nodes"] == 4


def test_traffic_from_the_committed_summary():
    t = bench.ncu_traffic("halo_kernel_moldyn_4M")
    algorithmic = 8 * 134230348 + 24 * 4194304
    assert t is not None and 0.5 * algorithmic < t < 1.5 * algorithmic
    assert bench.ncu_traffic("no_such_kernel") is None
