"""Batched instances (irr_batch_*): one persistent launch over many systems (GPU).

Each instance's result must be bitwise the result it has alone (same kernel
shape), through a plain step, a CUDA-graph replay and after autotuning (then
within the FP32 reordering tolerance, since the shape may change).
"""
import numpy as np
import pytest

from helpers import TOL_NORMWISE_F64, normwise_error

pytestmark = pytest.mark.gpu


def make_systems(count=12, seed=20260004):
    import workloads as W
    rng = np.random.Generator(np.random.PCG64(seed))
    sizes = np.exp(rng.uniform(np.log(1024), np.log(20000), count)).astype(int)
    out = []
    for k, n in enumerate(sizes):
        pos, side = W.random_box(int(n), 0.8442, seed + 10 + k)
        out.append((pos, side))
    return out


def handle_for(irr, pos, side, edges, **cfg):
    h = irr.Handle(irr.default_config(map_idx=irr.IRR_MAP_LJ_MOLDYN, exec=1, **cfg))
    h.set_params(irr.moldyn_params(side, 2.5))
    h.set_edges(edges)
    h.set_nodes(pos, 12)
    h.init()
    return h


def test_batch_equals_alone_bitwise(built_lib):
    import irregular_gb300 as irr
    systems = make_systems()
    alone, handles, lists = [], [], []
    for pos, side in systems:
        e = irr.neighbor_build(pos, side, 2.5 * 2.5).to_host()
        lists.append(e)
        h = handle_for(irr, pos, side, e)
        h.step()
        alone.append(h.get_result(elm_size=12).copy())
        handles.append(handle_for(irr, pos, side, e))
    b = irr.Batch()
    for h in handles:
        b.add(h)
    b.finalize(autotune=False)
    info = b.info()
    assert info.num_instances == len(systems)
    assert info.num_edges == sum(x.shape[0] for x in lists)
    b.step()
    b.sync()
    for h, ref in zip(handles, alone):
        assert np.array_equal(h.get_result(elm_size=12).view(np.uint32), ref.view(np.uint32))
    # graph replay, several steps
    b.capture()
    assert b.info().graph == 1
    for _ in range(3):
        b.step()
    b.sync()
    for h, ref in zip(handles, alone):
        assert np.array_equal(h.get_result(elm_size=12).view(np.uint32), ref.view(np.uint32))
    b.close()


def test_batch_after_autotune_matches_fp64(built_lib, oracle_lib):
    import irregular_gb300 as irr
    O = oracle_lib
    systems = make_systems(count=6, seed=77)
    handles, refs = [], []
    for pos, side in systems:
        e = irr.neighbor_build(pos, side, 2.5 * 2.5).to_host()
        f64, _ = O.lj_reduce_f64(pos.astype(np.float64), e, O.lj_param(6.25, side, True))
        refs.append(f64)
        handles.append(handle_for(irr, pos, side, e))
    b = irr.Batch()
    for h in handles:
        b.add(h)
    b.finalize(autotune=True)
    inf = b.info()
    assert inf.lanes_per_row in (4, 8, 16) and inf.block_nodes in (64, 256, 1024)
    b.step()
    b.sync()
    for h, f64 in zip(handles, refs):
        assert normwise_error(h.get_result(elm_size=12), f64) <= TOL_NORMWISE_F64
    b.close()


def test_single_handle_autotune(built_lib, oracle_lib):
    import irregular_gb300 as irr
    O = oracle_lib
    import workloads as W
    pos, side = W.random_box(30000, 0.8442, 5)
    e = irr.neighbor_build(pos, side, 6.25).to_host()
    h = handle_for(irr, pos, side, e)
    h.autotune()
    inf = h.info()
    assert inf.lanes_per_row in (4, 8, 16)
    h.step()
    f64, _ = O.lj_reduce_f64(pos.astype(np.float64), e, O.lj_param(6.25, side, True))
    assert normwise_error(h.get_result(elm_size=12), f64) <= TOL_NORMWISE_F64


def test_batch_rejects_mixed_boundaries_and_plain_handles(built_lib):
    import irregular_gb300 as irr
    import workloads as W
    pos, side = W.random_box(2000, 0.8442, 9)
    e = irr.neighbor_build(pos, side, 6.25).to_host()
    b = irr.Batch()
    b.add(handle_for(irr, pos, side, e))
    h_open = irr.Handle(irr.default_config(map_idx=irr.IRR_MAP_LJ_MINIMD, exec=1))
    h_open.set_params(irr.minimd_params(6.25))
    h_open.set_edges(e)
    h_open.set_nodes(pos, 12)
    with pytest.raises(irr.IrregularError) as ei:
        b.add(h_open)
    assert ei.value.status == irr.IRR_ERR_ARG
    h_plain = irr.Handle(irr.default_config(map_idx=0, exec=0))
    with pytest.raises(irr.IrregularError):
        b.add(h_plain)
    b.close()
