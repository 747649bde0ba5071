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
    collective is needed because every result row is owned by one shard).
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


def local_positions(shard: Shard, owned_pos: np.ndarray, received: Dict[int, np.ndarray]):
    """[owned rows, then halo] positions from the owned block and the peers' messages."""
    halo_pos = np.empty((shard.halo.shape[0],) + owned_pos.shape[1:], owned_pos.dtype)
    for q, ids in shard.recv_from.items():
        halo_pos[np.searchsorted(shard.halo, ids)] = received[q]
    return np.concatenate([owned_pos, halo_pos], axis=0)
