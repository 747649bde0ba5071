"""The batched workload at full size (GPU): 512 independent periodic LJ systems
of log-uniform size in [1,024, 262,144] atoms (seeded as the benchmark's), each
uniform-random in its own box at density 0.8442, cutoff 2.5, all reduced by ONE
persistent launch per step replayed from a CUDA graph, with the autotuned
kernel shape.

Checked on a sample of instances that includes the largest and the smallest:
  * each instance's result in the batch equals, bit for bit, the same handle
    stepped alone;
  * a seeded sample of each sampled instance's nodes (all of them for small
    instances) against the FP64 oracle and the reference's numerics, with the
    per-result error stated per quantile.
"""
import math

import numpy as np
import pytest

from helpers import (TOL_NORMWISE_F64, TOL_PERNODE_F64, TOL_RESULT_MAX, TOL_RESULT_P50,
                     TOL_VS_REFERENCE, result_error_summary, scaled_error)

pytestmark = pytest.mark.gpu

COUNT = 512
BENCH_SEED = 20260002   # the benchmark's seeds: sizes from + 2, instance k's positions from + 100 + k
SEED = BENCH_SEED + 2
CUTOFF = 2.5
RHO = 0.8442
NODE_SAMPLE = 1500


def test_512_instances(built_lib, oracle_lib):
    import irregular_gb300 as irr
    import workloads as W
    O = oracle_lib
    rng = np.random.Generator(np.random.PCG64(SEED))
    sizes = np.floor(np.exp(rng.uniform(math.log(1024), math.log(262144), COUNT))).astype(int)
    assert sizes.min() >= 1024 and sizes.max() <= 262144
    pick = {int(np.argmax(sizes)), int(np.argmin(sizes))}
    pick |= set(int(k) for k in np.random.Generator(np.random.PCG64(SEED + 1)).choice(
        COUNT, 6, replace=False))
    handles, keep = [], {}
    for k, n in enumerate(sizes):
        pos, side = W.random_box(int(n), RHO, BENCH_SEED + 100 + k)
        d_edges = irr.neighbor_build(pos, side, CUTOFF * CUTOFF)
        h = irr.Handle(irr.default_config(map_idx=irr.IRR_MAP_LJ_MOLDYN,
                                          exec=irr.IRR_EXEC_PARTITIONED))
        h.set_params(irr.moldyn_params(side, CUTOFF))
        h.set_edges(d_edges)
        h.set_nodes(pos, 12)
        h.init()
        if k in pick:
            keep[k] = (pos, side, d_edges.to_host())
        d_edges.close()
        handles.append(h)
    b = irr.Batch(0)
    for h in handles:
        b.add(h)
    b.finalize(autotune=True)
    b.capture()
    b.step()
    b.step()
    b.sync()
    inf = b.info()
    assert inf.num_instances == COUNT and inf.graph == 1
    batched = {k: handles[k].get_result(elm_size=12) for k in keep}
    for k, (pos, side, edges) in sorted(keep.items()):
        h = handles[k]
        h.step()
        alone = h.get_result(elm_size=12)
        assert np.array_equal(alone.view(np.uint32), batched[k].view(np.uint32)), k
        n = pos.shape[0]
        s = np.arange(n) if n <= NODE_SAMPLE else np.sort(
            np.random.Generator(np.random.PCG64(SEED + 1000 + k)).choice(n, NODE_SAMPLE,
                                                                          replace=False))
        sel = np.zeros(n, bool)
        sel[s] = True
        inc = edges[sel[edges[:, 0]] | sel[edges[:, 1]]]
        p = O.lj_param(CUTOFF * CUTOFF, side, True)
        pos64 = pos.astype(np.float64)
        f64, sabs = O.lj_reduce_f64(pos64, inc, p)
        sinf = O.lj_edge_scale_inf(pos64, inc, p)
        fref = O.lj_reduce_refnum(pos64, inc, p)
        f = batched[k][s]
        assert scaled_error(f, fref[s], sabs[s]) <= TOL_VS_REFERENCE, k
        assert np.abs(f - f64[s]).max() / np.abs(f64[s]).max() <= TOL_NORMWISE_F64, k
        assert scaled_error(f, f64[s], sabs[s]) <= TOL_PERNODE_F64, k
        err = result_error_summary(f, f64[s], sinf[s])
        assert err["p50"] <= TOL_RESULT_P50 and err["max"] <= TOL_RESULT_MAX, (k, err)
    b.close()
    for h in handles:
        h.close()
