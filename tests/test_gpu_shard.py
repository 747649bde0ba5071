"""Sharded execution on one GPU: the plan of sharding.py (owned row ranges of
the partition, halos, per-peer exchange lists) turned into one handle per
shard (irr_set_shard, irr_set_nodes_range), the halo exchanged through host
memory, the union of the shards' owned rows compared with one handle over the
whole problem -- the reference's per-rank view and its halo exchange
(moldyn/irregular/partition_view.cpp:44-282, 285-435) on a single device.

With the CSR or sliced layout each owned row holds the same neighbours in the
same order as in the whole-problem handle, so the union is equal bit for
bit; the staged layout sums a row in an order set by its work item's table,
so shards agree with the whole problem to the compensated-sum tolerance.
"""
import numpy as np
import pytest

import irregular_gb300 as irr
import sharding
from helpers import TOL_PERNODE_F64, load_golden, random_box, scaled_error

pytestmark = pytest.mark.gpu


def as_f4(pos):
    p = np.zeros((pos.shape[0], 4), np.float32)
    p[:, :3] = pos
    return p


def whole_handle(pos4, edges, params, layout):
    h = irr.Handle(exec=irr.IRR_EXEC_PARTITIONED, layout=layout)
    h.set_params(params)
    h.set_edges(edges)
    h.set_nodes(pos4, elm_size=16)
    h.init()
    return h


def shard_handles(plans, pos4_exec, params, layout):
    hs = []
    for lp in plans:
        h = irr.Handle(exec=irr.IRR_EXEC_PARTITIONED, layout=layout, reorder=0)
        h.set_params(params)
        h.set_shard(lp.own_lo, lp.own_hi)
        h.set_edges(lp.edges)
        h.set_nodes(pos4_exec[lp.nodes], elm_size=16)
        h.init()
        info = h.info()
        assert info.own_lo == lp.own_lo and info.own_hi == lp.own_hi
        # owned rows only: the entries of the shard's rows of the whole problem
        assert info.num_entries == int(np.diff(sharding.local_rows(lp)[0]).sum())
        hs.append(h)
    return hs


def exchange_through_host(plans, hs, owned_pos):
    """Every shard's halo from its peers' owned positions, over host memory:
    rank q sends owned_pos[q][send_local[r] - own_lo_q] to rank r, which
    writes them at its local ids recv_local[q]; then the halo ranges below and
    above the owned range are handed to the handle."""
    for lp, h in zip(plans, hs):
        n_local = lp.nodes.shape[0]
        buf = np.zeros((n_local, 4), np.float32)
        filled = np.zeros(n_local, bool)
        for q, ids in lp.recv_local.items():
            peer = plans[q]
            msg = owned_pos[q][peer.send_local[lp.rank] - peer.own_lo]
            buf[ids] = msg
            filled[ids] = True
        filled[lp.own_lo:lp.own_hi] = True
        assert filled.all()
        h.set_nodes_range(owned_pos[lp.rank], lp.own_lo, elm_size=16)
        if lp.own_lo > 0:
            h.set_nodes_range(buf[:lp.own_lo], 0, elm_size=16)
        if lp.own_hi < n_local:
            h.set_nodes_range(buf[lp.own_hi:], lp.own_hi, elm_size=16)


def union_of(plans, hs, n):
    out = np.zeros((n, 4), np.float32)
    for lp, h in zip(plans, hs):
        h.step()
        out[lp.lo:lp.hi] = h.get_result(elm_size=16)
    return out


def run_case(pos, edges, params, parts, layout, exact, O=None, side=None, rc2=None):
    pos4 = as_f4(pos)
    hw = whole_handle(pos4, edges, params, layout)
    perm, row_off, col = hw.partition()
    plans = [sharding.local_problem(sh, row_off, col) for sh in sharding.plan(row_off, col, parts)]
    assert sum(lp.hi - lp.lo for lp in plans) == pos.shape[0]
    hs = shard_handles(plans, pos4[perm], params, layout)

    def check(pos4_now):
        hw.set_nodes(pos4_now, elm_size=16)
        hw.step()
        whole = hw.get_result(elm_size=16)[perm]
        got = union_of(plans, hs, pos.shape[0])
        if exact:
            assert np.array_equal(got.view(np.uint32), whole.view(np.uint32))
        else:
            f64, sabs = O.lj_reduce_f64(pos4_now[:, :3].astype(np.float64), edges,
                                        O.lj_param(rc2, side, True))
            assert scaled_error(got[:, :3], f64[perm], sabs[perm]) <= TOL_PERNODE_F64
            assert scaled_error(got[:, :3], whole[:, :3], sabs[perm]) <= 2 * TOL_PERNODE_F64

    check(pos4)
    # a second step with moved nodes: owned positions from each rank, halos
    # exchanged through host memory
    rng = np.random.Generator(np.random.PCG64(5))
    moved = pos4.copy()
    moved[:, :3] += (rng.random((pos.shape[0], 3), dtype=np.float32) - 0.5) * np.float32(0.02)
    if side is not None:
        moved[:, :3] = np.mod(moved[:, :3], np.float32(side))
        moved[moved >= np.float32(side)] = 0.0
    moved_exec = moved[perm]
    exchange_through_host(plans, hs, [moved_exec[lp.lo:lp.hi] for lp in plans])
    check(moved)


@pytest.mark.parametrize("layout", [irr.IRR_LAYOUT_SLICED, irr.IRR_LAYOUT_CSR])
@pytest.mark.parametrize("parts", [2, 3])
@pytest.mark.parametrize("name", ["moldyn_random_2048", "moldyn_shuffled_dups_1500"])
def test_shards_equal_whole_problem_bitwise(built_lib, name, parts, layout):
    c = load_golden(name)
    params = irr.moldyn_params(float(c["side"]), float(c["cutoff"]))
    run_case(c["pos"].astype(np.float32), c["edges"], params, parts, layout, exact=True,
             side=float(c["side"]))


@pytest.mark.parametrize("parts", [2, 4])
def test_shards_random_box(built_lib, oracle_lib, parts):
    """65,536 nodes, ~64 neighbours: bitwise with the sliced layout, and the
    default (staged) layout within tolerance of the whole problem and FP64."""
    O = oracle_lib
    pos, L = random_box(65536, 32.0 / (4.0 / 3.0 * np.pi * 2.5 ** 3), 404)
    edges = O.neighbor_half_list(pos, float(L), np.float32(2.5 * 2.5))
    params = irr.moldyn_params(float(L), 2.5)
    run_case(pos, edges, params, parts, irr.IRR_LAYOUT_SLICED, exact=True, side=float(L))
    run_case(pos, edges, params, parts, irr.IRR_LAYOUT_AUTO, exact=False, O=O, side=float(L),
             rc2=2.5 * 2.5)


def test_shard_arguments(built_lib):
    c = load_golden("moldyn_random_2048")
    h = irr.Handle(exec=irr.IRR_EXEC_PARTITIONED)
    h.set_params(irr.moldyn_params(float(c["side"]), float(c["cutoff"])))
    h.set_edges(c["edges"])
    h.set_nodes(as_f4(c["pos"].astype(np.float32)), elm_size=16)
    with pytest.raises(irr.IrregularError):
        h.set_shard(10, 5)
    h.set_shard(0, 5000)  # beyond the node count: refused at init
    with pytest.raises(irr.IrregularError) as e:
        h.init()
    assert e.value.status == irr.IRR_ERR_STATE
    h2 = irr.Handle(exec=irr.IRR_EXEC_PARTITIONED)
    h2.set_params(irr.moldyn_params(float(c["side"]), float(c["cutoff"])))
    h2.set_edges(c["edges"])
    h2.set_nodes(as_f4(c["pos"].astype(np.float32)), elm_size=16)
    h2.init()
    with pytest.raises(irr.IrregularError) as e:
        h2.set_shard(0, 10)  # after init
    assert e.value.status == irr.IRR_ERR_STATE
    with pytest.raises(irr.IrregularError):
        h2.set_nodes_range(np.zeros((4, 4), np.float32), 2046, elm_size=16)  # past the end


def test_pipelined_steps_on_shards(built_lib):
    """irr_step_pipelined on shard handles returns the owned rows only, the
    bits of the sequential calls."""
    c = load_golden("moldyn_random_2048")
    params = irr.moldyn_params(float(c["side"]), float(c["cutoff"]))
    pos4 = as_f4(c["pos"].astype(np.float32))
    hw = whole_handle(pos4, c["edges"], params, irr.IRR_LAYOUT_SLICED)
    perm, row_off, col = hw.partition()
    plans = [sharding.local_problem(sh, row_off, col) for sh in sharding.plan(row_off, col, 2)]
    hs = shard_handles(plans, pos4[perm], params, irr.IRR_LAYOUT_SLICED)
    hw.step()
    whole = hw.get_result(elm_size=16)[perm]
    for lp, h in zip(plans, hs):
        recs = np.ascontiguousarray(pos4[perm][lp.nodes])
        outs = [np.empty((lp.own_hi - lp.own_lo, 4), np.float32) for _ in range(3)]
        for o in outs:
            h.step_pipelined(recs, o, 16, 16)
        h.pipeline_sync()
        for o in outs:
            assert np.array_equal(o.view(np.uint32), whole[lp.lo:lp.hi].view(np.uint32))


@pytest.mark.parametrize("layout", [irr.IRR_LAYOUT_AUTO, irr.IRR_LAYOUT_SLICED, irr.IRR_LAYOUT_CSR])
def test_degenerate_shards(built_lib, layout):
    """A shard that owns no rows, and one that owns every node but sees no
    edges: both run, and return no records / zero forces."""
    c = load_golden("moldyn_random_2048")
    params = irr.moldyn_params(float(c["side"]), float(c["cutoff"]))
    pos4 = as_f4(c["pos"].astype(np.float32))
    h = irr.Handle(exec=irr.IRR_EXEC_PARTITIONED, layout=layout, reorder=0)
    h.set_params(params)
    h.set_shard(5, 5)
    h.set_edges(c["edges"])
    h.set_nodes(pos4, elm_size=16)
    h.init()
    h.step()
    assert h.info().num_entries == 0
    assert h.get_result(elm_size=16).shape[0] == 0
    h2 = irr.Handle(exec=irr.IRR_EXEC_PARTITIONED, layout=layout, reorder=0)
    h2.set_params(params)
    h2.set_shard(0, pos4.shape[0])
    h2.set_edges(np.zeros((0, 2), np.int32))
    h2.set_nodes(pos4, elm_size=16)
    h2.init()
    h2.step()
    assert np.all(h2.get_result(elm_size=16) == 0)
