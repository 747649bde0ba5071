"""Sharding plan of the partitioned reduction across GPUs (host logic).

The reference splits the reduction space across MPI ranks: each rank owns a
range of nodes, keeps the edges touching them (cross edges on both sides) and
receives, every step, the positions of the remote nodes those edges read,
appended after its own nodes (moldyn/irregular/partition_view.cpp:44-282,
exchange :285-435; paper Fig. 3).  The owner-computes layout already holds
every edge in both endpoint rows, so a shard is a contiguous range of rows of
the partition; what a shard needs from the others is exactly the set of
neighbour ids outside its range -- its halo.  This module computes that plan:

  * shard ranges, cut so each shard holds about the same number of entries;
  * per shard: its halo (global ids, sorted), the local CSR whose columns
    index [owned nodes, then halo nodes], and for every peer the ids the peer
    must send (an all-to-all-v of positions per step; no reduction
    collective is needed because every result row is owned by one shard);
  * per shard, the local problem a handle reduces (irr_set_shard): its nodes
    in the whole problem's execution order, its owned range, the pairs that
    touch an owned node, and the local ids each exchange reads and writes.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, List

import numpy as np


@dataclass
class Shard:
    rank: int
    lo: int                      # owned rows [lo, hi) of the partition order
    hi: int
    halo: np.ndarray             # global ids of remote neighbours, sorted
    row_off: np.ndarray          # local CSR over the owned rows
    col: np.ndarray              # local ids: owned k -> k - lo, halo h -> (hi - lo) + index
    recv_from: Dict[int, np.ndarray] = field(default_factory=dict)  # peer -> global ids
    send_to: Dict[int, np.ndarray] = field(default_factory=dict)    # peer -> global ids


def shard_ranges(row_off: np.ndarray, parts: int) -> List[tuple]:
    """Contiguous row ranges with about equal entry counts."""
    n = row_off.shape[0] - 1
    total = int(row_off[-1])
    cuts = [0]
    for p in range(1, parts):
        target = total * p // parts
        cuts.append(int(np.searchsorted(row_off, target, side="left")))
    cuts.append(n)
    cuts = np.maximum.accumulate(np.clip(cuts, 0, n))
    return [(int(cuts[p]), int(cuts[p + 1])) for p in range(parts)]


def plan(row_off: np.ndarray, col: np.ndarray, parts: int) -> List[Shard]:
    row_off = np.asarray(row_off, np.int64)
    col = np.asarray(col, np.int64)
    ranges = shard_ranges(row_off, parts)
    shards = []
    for r, (lo, hi) in enumerate(ranges):
        cols = col[row_off[lo]:row_off[hi]]
        remote = (cols < lo) | (cols >= hi)
        halo = np.unique(cols[remote])
        local = np.empty_like(cols)
        local[~remote] = cols[~remote] - lo
        local[remote] = (hi - lo) + np.searchsorted(halo, cols[remote])
        sh = Shard(rank=r, lo=lo, hi=hi, halo=halo,
                   row_off=(row_off[lo:hi + 1] - row_off[lo]).astype(np.int64), col=local)
        for q, (qlo, qhi) in enumerate(ranges):
            if q != r:
                ids = halo[(halo >= qlo) & (halo < qhi)]
                if ids.size:
                    sh.recv_from[q] = ids
        shards.append(sh)
    for sh in shards:
        for q, ids in sh.recv_from.items():
            shards[q].send_to[sh.rank] = ids
    return shards


def half_edges_of_rows(row_off: np.ndarray, col: np.ndarray, lo: int, hi: int) -> np.ndarray:
    """The half edges (pairs listed once, both ids in execution order) whose
    directed entries fill rows [lo, hi) of the CSR: from each row r its
    entries c > r, its entries c outside [lo, hi) below r (their own rows are
    not in the range), and half of its entries c == r (a self pair fills its
    row twice).  Duplicated pairs keep their multiplicity."""
    row_off = np.asarray(row_off, np.int64)
    col = np.asarray(col, np.int64)
    rows = np.repeat(np.arange(lo, hi, dtype=np.int64), np.diff(row_off[lo:hi + 1]))
    cols = col[row_off[lo]:row_off[hi]]
    keep = (cols > rows) | ((cols < rows) & ((cols < lo) | (cols >= hi)))
    self_pair = cols == rows
    if np.any(self_pair):
        # every second self entry of each row
        idx = np.flatnonzero(self_pair)
        first = np.r_[True, rows[idx][1:] != rows[idx][:-1]]
        start = np.maximum.accumulate(np.where(first, np.arange(idx.size), 0))
        keep[idx[(np.arange(idx.size) - start) % 2 == 0]] = True
    return np.stack([rows[keep], cols[keep]], axis=1)


@dataclass
class LocalProblem:
    """One shard as a handle of its own (irr_set_shard): its nodes -- owned
    and halo -- in the whole problem's execution order, so that the owned ids
    form the contiguous local range [own_lo, own_hi) and every owned row keeps
    its neighbours in the same order."""
    rank: int
    lo: int
    hi: int
    nodes: np.ndarray            # global execution ids of the local nodes, ascending
    own_lo: int
    own_hi: int
    edges: np.ndarray            # (k, 2) int32 local ids: every pair touching an owned node, once
    send_local: Dict[int, np.ndarray] = field(default_factory=dict)  # peer -> local ids it needs
    recv_local: Dict[int, np.ndarray] = field(default_factory=dict)  # peer -> local ids it fills


def local_problem(shard: Shard, row_off: np.ndarray, col: np.ndarray) -> LocalProblem:
    nodes = np.union1d(np.arange(shard.lo, shard.hi, dtype=np.int64), shard.halo.astype(np.int64))
    own_lo = int(np.searchsorted(nodes, shard.lo))
    own_hi = own_lo + (shard.hi - shard.lo)
    half = half_edges_of_rows(row_off, col, shard.lo, shard.hi)
    edges = np.searchsorted(nodes, half).astype(np.int32)
    lp = LocalProblem(rank=shard.rank, lo=shard.lo, hi=shard.hi, nodes=nodes, own_lo=own_lo,
                      own_hi=own_hi, edges=edges)
    for q, ids in shard.send_to.items():
        lp.send_local[q] = (np.asarray(ids, np.int64) - shard.lo + own_lo).astype(np.int64)
    for q, ids in shard.recv_from.items():
        lp.recv_local[q] = np.searchsorted(nodes, ids).astype(np.int64)
    return lp


def local_rows(lp: LocalProblem):
    """CSR of the owned rows of a local problem (local ids, columns
    ascending): what a shard handle reduces."""
    e = lp.edges.astype(np.int64)
    r = np.concatenate([e[:, 0], e[:, 1]])
    c = np.concatenate([e[:, 1], e[:, 0]])
    own = (r >= lp.own_lo) & (r < lp.own_hi)
    r, c = r[own] - lp.own_lo, c[own]
    order = np.lexsort((c, r))
    r, c = r[order], c[order]
    n_own = lp.own_hi - lp.own_lo
    row_off = np.zeros(n_own + 1, np.int64)
    np.add.at(row_off, r + 1, 1)
    return np.cumsum(row_off), c


def local_positions(shard: Shard, owned_pos: np.ndarray, received: Dict[int, np.ndarray]):
    """[owned rows, then halo] positions from the owned block and the peers' messages."""
    halo_pos = np.empty((shard.halo.shape[0],) + owned_pos.shape[1:], owned_pos.dtype)
    for q, ids in shard.recv_from.items():
        halo_pos[np.searchsorted(shard.halo, ids)] = received[q]
    return np.concatenate([owned_pos, halo_pos], axis=0)


class HaloExchange:
    """The per-step halo exchange of one rank's local problem over
    torch.distributed point-to-point operations (NCCL between GPUs, gloo on
    CPU): the owned records each peer needs are packed by index, every send
    and receive is posted in one batch, and the received records are written
    at their local ids.  `local` is the rank's (n_local, width) record tensor
    in local order; run() leaves it with current halo records.  The
    reference's exchange_halo_node_data (partition_view.cpp:285-435) sends the
    same per-peer lists with MPI."""

    def __init__(self, lp: LocalProblem, device, width: int = 4, dtype=None):
        import torch

        dtype = dtype or torch.float32
        self.send = {q: torch.as_tensor(ids, dtype=torch.int64, device=device)
                     for q, ids in sorted(lp.send_local.items())}
        self.recv = {q: torch.as_tensor(ids, dtype=torch.int64, device=device)
                     for q, ids in sorted(lp.recv_local.items())}
        self.sbuf = {q: torch.empty((t.shape[0], width), dtype=dtype, device=device)
                     for q, t in self.send.items()}
        self.rbuf = {q: torch.empty((t.shape[0], width), dtype=dtype, device=device)
                     for q, t in self.recv.items()}

    @property
    def records(self) -> int:
        return sum(t.shape[0] for t in self.recv.values())

    def run(self, local):
        import torch
        import torch.distributed as dist

        for q, idx in self.send.items():
            torch.index_select(local, 0, idx, out=self.sbuf[q])
        ops = [dist.P2POp(dist.isend, self.sbuf[q], q) for q in self.send]
        ops += [dist.P2POp(dist.irecv, self.rbuf[q], q) for q in self.recv]
        if ops:
            for req in dist.batch_isend_irecv(ops):
                req.wait()
        for q, idx in self.recv.items():
            local.index_copy_(0, idx, self.rbuf[q])
