"""The benchmark workload at full size (GPU): 4,194,304 nodes, ~134.2M edges.

The FP64 oracle cannot reduce the whole list in a test's time budget, so the
full size is checked through what does not depend on size:
  * the GPU neighbour list's first rows equal the oracle's list rows, bit for bit;
  * a seeded sample of nodes, each with all its incident edges, matches the
    reference's numerics and the FP64 oracle within the stated tolerances;
  * CSR and sliced layouts give the same bits, and a second step repeats them;
  * Newton's third law: the total force vanishes to FP32 rounding;
  * the plain (atomic) path agrees with the partitioned path on the sample;
  * the caller's random node order (reorder = 0, no curve order) gives the
    same parity on the sample;
  * the per-result error against FP64 (helpers.result_errors) is stated per
    quantile.
"""
import math

import numpy as np
import pytest

from helpers import (TOL_NORMWISE_F64, TOL_PERNODE_F64, TOL_RESULT_MAX, TOL_RESULT_P50,
                     TOL_VS_REFERENCE, result_error_summary, scaled_error)

pytestmark = pytest.mark.gpu

N = 4194304
CUTOFF = 2.5
DENSITY = 64.0 / (4.0 / 3.0 * math.pi * CUTOFF ** 3)
SEED = 20260002   # the bench workload's seed
SAMPLE = 2000
LIST_ROWS = 4096


def workload():
    rng = np.random.Generator(np.random.PCG64(SEED))
    side = np.float32((N / DENSITY) ** (1.0 / 3.0))
    pos = (rng.random((N, 3), dtype=np.float32) * side).astype(np.float32)
    pos[pos >= side] = 0.0
    return pos, side


def run(irr, pos, side, d_edges, **cfg):
    h = irr.Handle(irr.default_config(map_idx=irr.IRR_MAP_LJ_MOLDYN, **cfg))
    h.set_params(irr.moldyn_params(float(side), CUTOFF))
    h.set_edges(d_edges)
    h.set_nodes(pos, 12)
    h.step()
    f = h.get_result(elm_size=12)
    return f, h


@pytest.fixture(scope="module")
def full(built_lib, oracle_lib):
    import irregular_gb300 as irr
    O = oracle_lib
    pos, side = workload()
    d_edges = irr.neighbor_build(pos, float(side), CUTOFF * CUTOFF)
    edges = d_edges.to_host()
    rng = np.random.Generator(np.random.PCG64(SEED + 1))
    sample = np.sort(rng.choice(N, SAMPLE, replace=False))
    sel = np.zeros(N, bool)
    sel[sample] = True
    incident = edges[sel[edges[:, 0]] | sel[edges[:, 1]]]
    pos64 = pos.astype(np.float64)
    p = O.lj_param(CUTOFF * CUTOFF, float(side), True)
    f64, sabs = O.lj_reduce_f64(pos64, incident, p)
    sinf = O.lj_edge_scale_inf(pos64, incident, p)
    fref = O.lj_reduce_refnum(pos64, incident, p)
    yield dict(irr=irr, O=O, pos=pos, side=side, d_edges=d_edges, edges=edges, sample=sample,
               f64=f64[sample], sabs=sabs[sample], sinf=sinf[sample], fref=fref[sample])
    d_edges.close()


def test_list_rows_match_oracle(full):
    O, pos, side, edges = full["O"], full["pos"], full["side"], full["edges"]
    assert 134_000_000 < edges.shape[0] < 134_500_000
    head = edges[edges[:, 0] < LIST_ROWS]
    ref = O.neighbor_half_list_rows(pos, float(side), np.float32(CUTOFF * CUTOFF), 0, LIST_ROWS)
    assert np.array_equal(head, ref)


def test_sample_parity_layouts_and_reproducibility(full):
    irr, pos, side, d_edges = full["irr"], full["pos"], full["side"], full["d_edges"]
    s, f64, sabs, fref = full["sample"], full["f64"], full["sabs"], full["fref"]
    f_sl, h_sl = run(irr, pos, side, d_edges, exec=irr.IRR_EXEC_PARTITIONED,
                     layout=irr.IRR_LAYOUT_SLICED)
    assert h_sl.info().layout == irr.IRR_LAYOUT_SLICED
    fs = f_sl[s]
    assert scaled_error(fs, fref, sabs) <= TOL_VS_REFERENCE
    assert np.abs(fs - f64).max() / np.abs(f64).max() <= TOL_NORMWISE_F64
    assert scaled_error(fs, f64, sabs) <= TOL_PERNODE_F64
    err = result_error_summary(fs, f64, full["sinf"])
    assert err["p50"] <= TOL_RESULT_P50 and err["max"] <= TOL_RESULT_MAX, err
    # a second step repeats the bits
    h_sl.step()
    assert np.array_equal(h_sl.get_result(elm_size=12).view(np.uint32), f_sl.view(np.uint32))
    h_sl.close()
    # the CSR layout gives the same sums in the same order
    f_csr, h_csr = run(irr, pos, side, d_edges, exec=irr.IRR_EXEC_PARTITIONED,
                       layout=irr.IRR_LAYOUT_CSR)
    assert h_csr.info().layout == irr.IRR_LAYOUT_CSR
    assert np.array_equal(f_csr, f_sl)
    h_csr.close()
    # Newton's third law: every edge adds +c to one row and -c (bit for bit)
    # to the other, so the total force is the rows' FP32 rounding only.  Uniform
    # random positions put a few pairs very close (|c| up to ~1e33), and those
    # rows dominate both the total and the scale sum(|f_i|).
    f64sum = f_sl.astype(np.float64)
    total = np.abs(f64sum.sum(axis=0))
    assert np.all(np.isfinite(total))
    assert np.all(total <= 1e-6 * np.abs(f64sum).sum(axis=0))


def test_caller_random_order(full):
    """reorder = 0, the workload's other node order (it is measured in both):
    blocks cut from the caller's random order, no curve order.  Each row sums
    the same terms (in the order of the caller's column ids), so the sample
    meets the same bounds, and a second step repeats the bits."""
    irr, pos, side, d_edges = full["irr"], full["pos"], full["side"], full["d_edges"]
    s, f64, sabs, fref = full["sample"], full["f64"], full["sabs"], full["fref"]
    f, h = run(irr, pos, side, d_edges, exec=irr.IRR_EXEC_PARTITIONED, reorder=0)
    perm, _, _ = h.partition(with_entries=False)
    assert np.array_equal(perm, np.arange(N, dtype=np.int32))
    fs = f[s]
    assert scaled_error(fs, fref, sabs) <= TOL_VS_REFERENCE
    assert np.abs(fs - f64).max() / np.abs(f64).max() <= TOL_NORMWISE_F64
    assert scaled_error(fs, f64, sabs) <= TOL_PERNODE_F64
    err = result_error_summary(fs, f64, full["sinf"])
    assert err["p50"] <= TOL_RESULT_P50 and err["max"] <= TOL_RESULT_MAX, err
    h.step()
    assert np.array_equal(h.get_result(elm_size=12).view(np.uint32), f.view(np.uint32))
    h.close()


def test_plain_path_agrees(full):
    irr, pos, side, d_edges = full["irr"], full["pos"], full["side"], full["d_edges"]
    s, f64, sabs = full["sample"], full["f64"], full["sabs"]
    f_pl, h = run(irr, pos, side, d_edges, exec=irr.IRR_EXEC_PLAIN)
    assert scaled_error(f_pl[s], f64, sabs) <= TOL_PERNODE_F64
    h.close()
