"""The staged ("halo") layout and the kernel that reads it (GPU).

  * the layout the GPU builds equals the oracle's restatement bit for bit
    (items, slice offsets, words, tables) -- integer work;
  * the reduction over it matches the reference's numerics and the FP64
    oracle within the same bounds as the other layouts (its rows sum their
    entries in the layout's bank-spreading order, so its bits differ from the
    CSR / sliced result's in the last places), repeats its own bits, and gives
    the same bits from a second handle;
  * limits: a graph with a hub row is refused (IRR_ERR_CAPACITY), and the
    layout needs 4 lanes per row;
  * the bounded-wait failure path and node-data resets work on this kernel too.
"""
import numpy as np
import pytest

from helpers import (TOL_NORMWISE_F64, TOL_PERNODE_F64, TOL_RESULT_MAX, TOL_RESULT_P50,
                     TOL_VS_REFERENCE, golden_names, load_golden, map_idx_of, normwise_error,
                     oracle_param, random_box, result_error_summary, scaled_error)

pytestmark = pytest.mark.gpu

RHO64 = 64.0 / (4.0 / 3.0 * np.pi * 2.5 ** 3)


def staged_handle(irr, case, **cfg):
    h = irr.Handle(irr.default_config(map_idx=map_idx_of(case), exec=irr.IRR_EXEC_PARTITIONED,
                                      layout=irr.IRR_LAYOUT_STAGED, **cfg))
    h.set_params(case["param"])
    h.set_edges(case["edges"])
    h.set_nodes(case["pos"], 24)
    h.init()
    assert h.info().layout == irr.IRR_LAYOUT_STAGED
    return h


def random_case(O, n, seed):
    pos, side = random_box(n, RHO64, seed)
    edges = O.neighbor_half_list(pos, float(side), np.float32(6.25))
    return {"pos": pos.astype(np.float64), "edges": edges, "param": np.array([side, 2.5]),
            "map": np.array("moldyn"), "side": np.float64(side), "cutoff": np.float64(2.5)}


def assert_layout_matches_oracle(O, h):
    _, row_off, col = h.partition()
    ref = O.staged_layout(row_off, col)
    got = h.staged()
    assert ref is not None
    for key in ("items", "slice_off", "words", "ids"):
        assert np.array_equal(got[key], ref[key]), key


@pytest.mark.parametrize("name", golden_names())
def test_layout_bit_exact(built_lib, oracle_lib, name):
    import irregular_gb300 as irr
    h = staged_handle(irr, load_golden(name))
    assert_layout_matches_oracle(oracle_lib, h)
    h.close()


def test_layout_bit_exact_random_box(built_lib, oracle_lib):
    import irregular_gb300 as irr
    h = staged_handle(irr, random_case(oracle_lib, 65536, 31))
    assert_layout_matches_oracle(oracle_lib, h)
    h.close()


@pytest.mark.parametrize("name", golden_names())
def test_parity_golden(built_lib, oracle_lib, name):
    import irregular_gb300 as irr
    O = oracle_lib
    c = load_golden(name)
    h = staged_handle(irr, c)
    h.step()
    f = h.get_result(elm_size=12)
    f64, sabs = O.lj_reduce_f64(c["pos"], c["edges"], oracle_param(O, c))
    assert scaled_error(f, c["f_ref"], sabs) <= TOL_VS_REFERENCE
    assert normwise_error(f, f64) <= TOL_NORMWISE_F64
    assert scaled_error(f, f64, sabs) <= TOL_PERNODE_F64
    # its own bits again, and from another handle
    h.step()
    assert np.array_equal(h.get_result(elm_size=12).view(np.uint32), f.view(np.uint32))
    h.close()
    h2 = staged_handle(irr, c)
    h2.step()
    assert np.array_equal(h2.get_result(elm_size=12).view(np.uint32), f.view(np.uint32))
    h2.close()


def test_random_box_parity(built_lib, oracle_lib):
    import irregular_gb300 as irr
    O = oracle_lib
    c = random_case(O, 65536, 32)
    h = staged_handle(irr, c)
    h.step()
    f = h.get_result(elm_size=12)
    p = oracle_param(O, c)
    f64, sabs = O.lj_reduce_f64(c["pos"], c["edges"], p)
    sinf = O.lj_edge_scale_inf(c["pos"], c["edges"], p)
    fref = O.lj_reduce_refnum(c["pos"], c["edges"], p)
    assert scaled_error(f, fref, sabs) <= TOL_VS_REFERENCE
    assert normwise_error(f, f64) <= TOL_NORMWISE_F64
    assert scaled_error(f, f64, sabs) <= TOL_PERNODE_F64
    err = result_error_summary(f, f64, sinf)
    assert err["p50"] <= TOL_RESULT_P50 and err["max"] <= TOL_RESULT_MAX, err
    # new node data (reset_node_data) through the same layout
    side32 = np.float32(c["side"])
    p2 = ((c["pos"].astype(np.float32) + np.float32(0.01)) % side32).astype(np.float32)
    p2[p2 >= side32] = 0.0  # float positions, as the kernel computes with them
    c2 = dict(c, pos=p2.astype(np.float64))
    h.set_nodes(c2["pos"], 24)
    h.step()
    g = h.get_result(elm_size=12)
    g64, gabs = O.lj_reduce_f64(c2["pos"], c["edges"], p)
    assert scaled_error(g, g64, gabs) <= TOL_PERNODE_F64
    h.close()


def test_hub_is_refused_and_lanes_checked(built_lib):
    import irregular_gb300 as irr
    n = 2000
    c = {"pos": np.random.default_rng(2).random((n, 3)) * 10.0,
         "edges": np.stack([np.zeros(n - 1, np.int32), np.arange(1, n, dtype=np.int32)], 1),
         "param": np.array([10.0, 2.5]), "map": np.array("moldyn")}
    with pytest.raises(irr.IrregularError) as ei:
        staged_handle(irr, c)
    assert ei.value.status == irr.IRR_ERR_CAPACITY
    c = load_golden("moldyn_random_2048")
    with pytest.raises(irr.IrregularError) as ei:
        staged_handle(irr, c, lanes_per_row=8)
    assert ei.value.status == irr.IRR_ERR_ARG


def test_wait_time_out_is_reported_and_recovers(built_lib):
    import irregular_gb300 as irr
    c = load_golden("moldyn_random_2048")
    h = staged_handle(irr, c)
    h.step()
    expect = h.get_result(elm_size=12)
    h.set_wait_limit(2000, withhold_once=True)
    h.step()
    with pytest.raises(irr.IrregularError) as ei:
        h.sync()
    assert ei.value.status == irr.IRR_ERR_DEVICE
    h.step()
    assert np.array_equal(h.get_result(elm_size=12).view(np.uint32), expect.view(np.uint32))
    h.close()
