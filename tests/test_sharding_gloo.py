"""The multi-GPU sharding plan, exercised by world_size-2 gloo ranks on CPU.

Each rank builds the local problem a shard handle reduces (sharding.
local_problem: its nodes in the whole problem's execution order, its owned
range, the pairs touching an owned node), receives its halo positions from
the other rank by the plan's exchange lists (point-to-point, the
all-to-all-v of the plan), and reduces its owned rows with the FP64 law;
rank 0 gathers the rows.  The union must equal the single-process reduction
of the whole edge list bit for bit.  tests/test_gpu_shard.py runs the same
local problems through shard handles on the GPU.
"""
import os
import socket

import numpy as np
import pytest

from helpers import load_golden

torch = pytest.importorskip("torch")
dist = pytest.importorskip("torch.distributed")


def lj_rows(pos, row_off, col, side, rc2):
    """FP64 owner-computes reduction of CSR rows (moldyn's law, minimum image)."""
    n = row_off.shape[0] - 1
    f = np.zeros((n, 3))
    for i in range(n):
        js = col[row_off[i]:row_off[i + 1]]
        if js.size == 0:
            continue
        d = pos[i] - pos[js]
        d = np.where(d < -0.5 * side, d + side, d)
        d = np.where(d > 0.5 * side, d - side, d)
        rd = (d * d).sum(axis=1)
        ok = rd < rc2
        r = 1.0 / rd[ok]
        s = r ** 7 - 0.5 * r ** 4
        f[i] = (d[ok] * s[:, None]).sum(axis=0)
    return f


def partition_of(case):
    from oracle import oracle as O
    pos32 = case["pos"].astype(np.float32)
    lo, scale = O.morton_frame(pos32)
    perm, inv, row_off, col = O.partition(pos32, lo, scale, case["edges"])
    return perm, row_off, col


def lj_owned_rows(pos_local, lp, side, rc2):
    """The owned rows of a local problem (sharding.local_rows), FP64."""
    row_off, col = sharding_mod().local_rows(lp)
    n_own = lp.own_hi - lp.own_lo
    f = np.zeros((n_own, 3))
    for i in range(n_own):
        js = col[row_off[i]:row_off[i + 1]]
        if js.size == 0:
            continue
        d = pos_local[lp.own_lo + i] - pos_local[js]
        d = np.where(d < -0.5 * side, d + side, d)
        d = np.where(d > 0.5 * side, d - side, d)
        rd = (d * d).sum(axis=1)
        ok = rd < rc2
        r = 1.0 / rd[ok]
        s = r ** 7 - 0.5 * r ** 4
        f[i] = (d[ok] * s[:, None]).sum(axis=0)
    return f


def sharding_mod():
    import sharding
    return sharding


def worker(rank, world, port, name, out_path):
    """One rank: the local problem a shard handle would get (irr_set_shard),
    its halo received from the peers by the exchange lists of the plan, its
    owned rows reduced; rank 0 gathers the rows."""
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sharding = sharding_mod()
    case = load_golden(name)
    perm, row_off, col = partition_of(case)
    pos = case["pos"][perm]                 # partition order
    side = float(case["side"])
    shards = sharding.plan(row_off, col, world)
    lps = [sharding.local_problem(sh, row_off, col) for sh in shards]
    me = lps[rank]
    # local positions: owned from this rank's own data, halo from the peers
    local = np.full((me.nodes.shape[0], 3), np.nan)
    local[me.own_lo:me.own_hi] = pos[me.lo:me.hi]
    owned = pos[me.lo:me.hi]
    reqs = []
    for q, ids in me.send_local.items():
        reqs.append(dist.isend(torch.from_numpy(owned[ids - me.own_lo].copy()), dst=q))
    for q, ids in me.recv_local.items():
        buf = torch.empty((ids.shape[0], 3), dtype=torch.float64)
        dist.recv(buf, src=q)
        local[ids] = buf.numpy()
    for r in reqs:
        r.wait()
    assert not np.isnan(local).any()
    f_own = lj_owned_rows(local, me, side, float(case["cutoff"]) ** 2)
    # gather owned rows on rank 0
    sizes = [s.hi - s.lo for s in shards]
    if rank == 0:
        full = np.zeros((pos.shape[0], 3))
        full[me.lo:me.hi] = f_own
        for q in range(1, world):
            buf = torch.empty((sizes[q], 3), dtype=torch.float64)
            dist.recv(buf, src=q)
            full[shards[q].lo:shards[q].hi] = buf.numpy()
        np.save(out_path, full)
    else:
        dist.send(torch.from_numpy(f_own), dst=0)
    dist.barrier()
    dist.destroy_process_group()


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def exchange_worker(rank, world, port, name, out_path):
    """sharding.HaloExchange (the bench's per-step exchange) on gloo: every
    rank's local record tensor, owned part filled, halo part NaN, must come out
    equal to the whole problem's records at the local nodes."""
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sharding = sharding_mod()
    case = load_golden(name)
    perm, row_off, col = partition_of(case)
    pos = np.zeros((perm.shape[0], 4), np.float32)
    pos[:, :3] = case["pos"][perm]
    lps = [sharding.local_problem(sh, row_off, col) for sh in sharding.plan(row_off, col, world)]
    me = lps[rank]
    local = torch.full((me.nodes.shape[0], 4), float("nan"))
    local[me.own_lo:me.own_hi] = torch.from_numpy(pos[me.lo:me.hi])
    hx = sharding.HaloExchange(me, "cpu")
    for _ in range(2):  # the buffers are reused step after step
        hx.run(local)
    ok = bool(np.array_equal(local.numpy(), pos[me.nodes]))
    flags = torch.tensor([1 if ok else 0], dtype=torch.int64)
    dist.all_reduce(flags)
    if rank == 0:
        np.save(out_path, flags.numpy())
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_halo_exchange_fills_every_halo(tmp_path, world):
    import torch.multiprocessing as mp
    out = str(tmp_path / "ok.npy")
    mp.start_processes(exchange_worker, args=(world, free_port(), "moldyn_random_2048", out),
                       nprocs=world, join=True, start_method="spawn")
    assert int(np.load(out)[0]) == world


@pytest.mark.parametrize("name", ["moldyn_random_2048", "moldyn_fcc_864"])
def test_two_rank_sharded_reduction_equals_single(oracle_lib, tmp_path, name):
    import torch.multiprocessing as mp
    out = str(tmp_path / "f.npy")
    mp.start_processes(worker, args=(2, free_port(), name, out), nprocs=2, join=True,
                       start_method="spawn")
    full = np.load(out)
    case = load_golden(name)
    perm, row_off, col = partition_of(case)
    ref = lj_rows(case["pos"][perm], row_off, col, float(case["side"]),
                  float(case["cutoff"]) ** 2)
    assert np.array_equal(full, ref)
    # and the single-process FP64 oracle agrees (partition order)
    O = oracle_lib
    f64, _ = O.lj_reduce_f64(case["pos"], case["edges"],
                              O.lj_param(float(case["cutoff"]) ** 2, float(case["side"]), True))
    assert np.abs(full - f64[perm]).max() <= 1e-9 * np.abs(f64).max()


def test_plan_properties():
    import sharding
    case = load_golden("moldyn_shuffled_dups_1500")
    _, row_off, col = partition_of(case)
    for parts in (2, 3, 4):
        shards = sharding.plan(row_off, col, parts)
        assert shards[0].lo == 0 and shards[-1].hi == row_off.shape[0] - 1
        assert all(a.hi == b.lo for a, b in zip(shards, shards[1:]))
        for sh in shards:
            assert np.all((sh.halo < sh.lo) | (sh.halo >= sh.hi))
            got = np.concatenate([ids for ids in sh.recv_from.values()]) if sh.recv_from else []
            assert np.array_equal(np.sort(got), sh.halo)
            for q, ids in sh.send_to.items():
                assert np.all((ids >= sh.lo) & (ids < sh.hi))
        counts = [int(row_off[s.hi] - row_off[s.lo]) for s in shards]
        # each cut lands within one row of its target
        assert max(counts) - min(counts) <= 2 * int(np.diff(row_off).max())


def test_local_problems_keep_every_owned_row(oracle_lib):
    """sharding.local_problem: every owned row of every shard holds, in local
    ids, exactly the whole problem's row -- with duplicated pairs and self
    pairs (which fill their row twice) kept."""
    import sharding
    O = oracle_lib
    rng = np.random.default_rng(3)
    n = 400
    pos = rng.random((n, 3)).astype(np.float32)
    e = rng.integers(0, n, (3000, 2)).astype(np.int32)
    e[:60, 1] = e[:60, 0]                        # self pairs
    e = np.concatenate([e, e[:150], e[:30]])     # duplicates, self pairs among them
    lo, scale = O.morton_frame(pos)
    _, _, row_off, col = O.partition(pos, lo, scale, e)
    for parts in (1, 2, 3, 5):
        for sh in sharding.plan(row_off, col, parts):
            lp = sharding.local_problem(sh, row_off, col)
            assert np.all(np.diff(lp.nodes) > 0)
            assert np.array_equal(lp.nodes[lp.own_lo:lp.own_hi], np.arange(sh.lo, sh.hi))
            ro, cc = sharding.local_rows(lp)
            assert np.array_equal(ro, row_off[sh.lo:sh.hi + 1] - row_off[sh.lo])
            assert np.array_equal(lp.nodes[cc], col[row_off[sh.lo]:row_off[sh.hi]])
            # the exchange lists cover the halo exactly once
            got = np.sort(np.concatenate([v for v in lp.recv_local.values()])) if lp.recv_local else []
            halo = np.r_[np.arange(0, lp.own_lo), np.arange(lp.own_hi, lp.nodes.shape[0])]
            assert np.array_equal(got, halo)


def test_plan_edge_cases():
    """More shards than rows (some shards own nothing), and a graph with no
    entries: the shards still tile the rows in order, empty shards have no
    halo and an empty local problem, and every owned row is kept."""
    import sharding
    row_off = np.array([0, 2, 3, 5, 6, 6], np.uint32)
    col = np.array([1, 2, 0, 0, 4, 2], np.int32)
    for parts in (1, 3, 5, 8):
        shards = sharding.plan(row_off, col, parts)
        assert len(shards) == parts
        assert shards[0].lo == 0 and shards[-1].hi == 5
        assert all(a.hi == b.lo for a, b in zip(shards, shards[1:]))
        for sh in shards:
            lp = sharding.local_problem(sh, row_off, col)
            if sh.hi == sh.lo:
                assert sh.halo.size == 0 and lp.nodes.size == 0
                continue
            ro, cc = sharding.local_rows(lp)
            assert np.array_equal(lp.nodes[cc], col[row_off[sh.lo]:row_off[sh.hi]])
    empty = sharding.plan(np.zeros(4, np.uint32), np.zeros(0, np.int32), 3)
    assert [(s.lo, s.hi) for s in empty][-1][1] == 3
    assert all(s.halo.size == 0 for s in empty)
