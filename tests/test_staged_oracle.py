"""The staged ("halo") entry layout as the oracle states it (CPU): the
properties the GPU kernel relies on, on a curve-ordered random box.

  * items cover the slices in order, each within the limits (8 slices, 3,584
    words, 640 table ids), and every prefix cut is the longest that fits;
  * each item's table is its rows' and their neighbours' ids, sorted, distinct;
  * every row of an item appears in exactly one of its slices, longest rows
    first, and the slices pad less than slices of 8 consecutive rows would;
  * each row's header gives its own table slot, its length and its index in
    the item, its first `len` picks are exactly its neighbours (as a
    multiset) and the rest are its own slot;
  * the bank-group order keeps a quarter-warp's 8 128-bit table loads at ~5.4
    shared-memory wavefronts (8 at random would be ~9).
"""
import numpy as np
import pytest

from helpers import random_box

N = 16384
RHO = 64.0 / (4.0 / 3.0 * np.pi * 2.5 ** 3)


@pytest.fixture(scope="module")
def case(oracle_lib):
    O = oracle_lib
    pos, side = random_box(N, RHO, 4242)
    edges = O.neighbor_half_list(pos, float(side), np.float32(6.25))
    lo, scale = O.morton_frame(pos)
    _, _, row_off, col = O.partition(pos, lo, scale, edges, curve="hilbert")
    return O, row_off, col, O.staged_layout(row_off, col)


def table_of(row_off, col, r0, r1):
    parts = [np.arange(r0, r1)] + [col[row_off[r]:row_off[r + 1]] for r in range(r0, r1)]
    return np.unique(np.concatenate(parts))


def test_items_cover_and_cut(case):
    O, row_off, col, L = case
    it, so = L["items"], L["slice_off"].astype(np.int64)
    n = row_off.shape[0] - 1
    assert it[0, 0] == 0 and it[-1, 0] + it[-1, 1] == n
    assert np.all(it[1:, 0] == it[:-1, 0] + it[:-1, 1])
    assert np.all(it[:, 1] <= 64) and np.all(it[:, 3] <= 3584) and np.all(it[:, 5] <= 640)
    assert np.all(it[:, 2] == so[it[:, 0] // 8])
    assert np.all(it[1:, 4] == it[:-1, 4] + it[:-1, 5])
    for k in range(0, it.shape[0], 17):
        row0, nrows, w0, nw, t0, nt = it[k]
        tab = L["ids"][t0:t0 + nt]
        assert np.array_equal(tab, table_of(row_off, col, row0, row0 + nrows))
        # the cut is the longest prefix that fits (unless the run ended there)
        end = row0 + nrows
        if nrows < 64 and end < n and k + 1 < it.shape[0]:
            q1 = end // 8 + 1
            more = table_of(row_off, col, row0, min(8 * q1, n)).shape[0] > 640
            words_more = so[q1] - so[row0 // 8] > 3584
            assert more or words_more or (end % 64 == 0)


def test_rows_reconstruct_and_banks(case):
    O, row_off, col, L = case
    it, so, w, ids = L["items"], L["slice_off"].astype(np.int64), L["words"], L["ids"]
    deg = np.diff(row_off)
    wf = lds = 0
    for k in range(0, it.shape[0], 7):
        row0, nrows, w0, nw, t0, nt = it[k]
        tab = ids[t0:t0 + nt]
        seen = []
        for q in range(row0 // 8, (row0 + nrows + 7) // 8):
            T = (so[q + 1] - so[q]) // 32 - 1
            sw = w[so[q]:so[q + 1]].reshape(T + 1, 32)
            lens = []
            for i in range(8):
                hdr = sw[0, 4 * i:4 * i + 4]
                assert np.all(hdr == hdr[0])
                h0 = int(hdr[0])
                if h0 == 1 << 31:  # a padding row
                    continue
                own, ln, lrow = (h0 & 0x3FFF) // 16, (h0 >> 14) & 0x3FF, (h0 >> 24) & 0x3F
                r = row0 + lrow
                seen.append(r)
                lens.append(ln)
                assert tab[own] == r and ln == row_off[r + 1] - row_off[r]
                picks = [((int(sw[t + 1, 4 * i + l]) >> (16 * h)) & 0xFFFF) // 16
                         for t in range(T) for h in range(2) for l in range(4)]
                assert sorted(tab[picks[:ln]].tolist()) == sorted(col[row_off[r]:row_off[r + 1]].tolist())
                assert all(p == own for p in picks[ln:])
            assert lens == sorted(lens, reverse=True) and T == (max(lens) + 7) // 8
            for t in range(T):
                for h in range(2):
                    for ph in range(4):
                        a = np.unique([(int(sw[t + 1, 8 * ph + j]) >> (16 * h)) & 0xFFFF
                                       for j in range(8)]) // 16
                        wf += max(1, np.bincount(a % 8, minlength=8).max())
                    lds += 1
        assert sorted(seen) == list(range(row0, row0 + nrows))
    assert wf / lds < 6.0, wf / lds
    # padding: slots over entries, against slices of 8 consecutive rows
    slots = 2 * (int(so[-1]) - 32 * (so.shape[0] - 1))
    consecutive = sum(64 * ((deg[r:r + 8].max() + 7) // 8) for r in range(0, deg.shape[0], 8))
    assert slots / deg.sum() < 1.12 and slots < 0.95 * consecutive, (slots / deg.sum(), consecutive / deg.sum())


def test_layout_does_not_apply_to_a_hub(oracle_lib):
    """A row longer than a slice's word budget allows (32 (T + 1) > 3,584
    words: ~880 entries) makes the layout inapplicable (None)."""
    O = oracle_lib
    n = 2000
    edges = np.stack([np.zeros(n - 1, np.int32), np.arange(1, n, dtype=np.int32)], 1)
    pos = np.random.default_rng(1).random((n, 3)).astype(np.float32)
    lo, scale = O.morton_frame(pos)
    _, _, row_off, col = O.partition(pos, lo, scale, edges)
    assert O.staged_layout(row_off, col) is None
