"""The multi-GPU sharding plan, exercised by world_size-2 gloo ranks on CPU.

Each rank owns a contiguous range of the partition's rows, receives its halo
positions from the other rank (point-to-point, the all-to-all-v of the plan),
and reduces its own rows with the FP64 law; rank 0 gathers the rows.  The
union must equal the single-process reduction of the whole edge list.
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


def worker(rank, world, port, name, out_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sharding
    case = load_golden(name)
    perm, row_off, col = partition_of(case)
    pos = case["pos"][perm]                 # partition order
    side = float(case["side"])
    shards = sharding.plan(row_off, col, world)
    me = shards[rank]
    # halo exchange: send what peers need, receive ours
    reqs, recv = [], {}
    for q, ids in me.send_to.items():
        reqs.append(dist.isend(torch.from_numpy(pos[ids].copy()), dst=q))
    for q, ids in me.recv_from.items():
        buf = torch.empty((ids.shape[0], 3), dtype=torch.float64)
        dist.recv(buf, src=q)
        recv[q] = buf.numpy()
    for r in reqs:
        r.wait()
    local = sharding.local_positions(me, pos[me.lo:me.hi], recv)
    f_own = lj_rows(local, me.row_off, me.col, side, float(case["cutoff"]) ** 2)
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
