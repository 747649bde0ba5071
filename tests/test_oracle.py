"""The CPU oracle, pinned against the reference's own outputs (CPU only).

The golden fixtures hold results of the reference's compiled CPU code
(tests/golden/make_golden.py); the known-answer neighbour counts are the
list sizes the reference logs (miniMD/2:13, moldyn/irresult/2:5).
"""
import numpy as np
import pytest

from helpers import (TOL_VS_REFERENCE, golden_names, load_golden, normwise_error, oracle_param,
                     random_box, scaled_error)


@pytest.mark.parametrize("name", golden_names())
def test_restatement_matches_reference_bitwise(oracle_lib, name):
    """irr_oracle.c's FP64-edge / FP32-accumulate numerics equal FCPU::map's bit for bit."""
    O = oracle_lib
    c = load_golden(name)
    f = O.lj_reduce_refnum(c["pos"], c["edges"], oracle_param(O, c))
    assert np.array_equal(f.view(np.uint32), c["f_ref"].view(np.uint32))


@pytest.mark.parametrize("name", golden_names())
def test_executor_port_matches_reference_executor(oracle_lib, name):
    """The ported pthread executor agrees with the reference's compute_cpu."""
    O = oracle_lib
    c = load_golden(name)
    p = oracle_param(O, c)
    f, secs = O.cpu_executor(c["pos"], c["edges"], p, threads=4, chunk=1000)
    f64, sabs = O.lj_reduce_f64(c["pos"], c["edges"], p)
    assert secs >= 0
    assert scaled_error(f, c["f_exec"], sabs) <= TOL_VS_REFERENCE
    assert scaled_error(f, f64, sabs) <= TOL_VS_REFERENCE


@pytest.mark.parametrize("name", golden_names())
def test_fp64_oracle_close_to_reference(oracle_lib, name):
    O = oracle_lib
    c = load_golden(name)
    f64, sabs = O.lj_reduce_f64(c["pos"], c["edges"], oracle_param(O, c))
    assert normwise_error(c["f_ref"], f64) <= 1e-6
    assert scaled_error(c["f_ref"], f64, sabs) <= TOL_VS_REFERENCE


def test_newton_third_law_fp64(oracle_lib):
    O = oracle_lib
    c = load_golden("moldyn_random_2048")
    f64, sabs = O.lj_reduce_f64(c["pos"], c["edges"], oracle_param(O, c))
    assert np.abs(f64.sum(axis=0)).max() <= 1e-9 * sabs.sum()


def test_neighbor_list_brute_force(oracle_lib):
    """The cell-binned list equals the O(n^2) definition on a small box."""
    O = oracle_lib
    pos, L = random_box(600, 0.5, 7)
    cut2 = np.float32(2.5 * 2.5)
    e = O.neighbor_half_list(pos, float(L), cut2)
    ref = []
    h = np.float32(0.5) * L
    for i in range(600):
        d = pos[i] - pos[i + 1:]
        d = np.where(d > h, d - L, np.where(d < -h, d + L, d)).astype(np.float32)
        sq = d * d
        r2 = (sq[:, 0] + sq[:, 1]) + sq[:, 2]
        for j in np.nonzero(r2 <= cut2)[0]:
            ref.append((i, i + 1 + j))
    assert np.array_equal(e, np.array(ref, np.int32).reshape(-1, 2))


def test_known_answer_minimd_neighbor_count(oracle_lib):
    """miniMD lj.in: FCC 50^3, rho 0.8442, cutneigh 2.8, no PBC -> 18,816,288 (miniMD/2:13)."""
    O = oracle_lib
    pos = O.fcc_minimd(50, 50, 50, 0.8442).astype(np.float32)
    assert pos.shape[0] == 500000
    assert O.neighbor_count(pos, 0.0, np.float32(2.8 * 2.8)) == 18816288


def test_known_answer_minimd_periodic_neighbor_count(oracle_lib):
    """miniMD's lattice with periodic images: 78 neighbours per atom inside
    2.8 (FCC shells 1-5; shell 6 is at 2.91), 39 per atom in the half list."""
    O = oracle_lib
    pos = O.fcc_minimd(50, 50, 50, 0.8442).astype(np.float32)
    side = float(np.float32(50 * (4 / 0.8442) ** (1 / 3)))
    assert O.neighbor_count(pos, side, np.float32(2.8 * 2.8)) == 19500000


@pytest.mark.slow
def test_known_answer_moldyn_neighbor_count(oracle_lib):
    """moldyn: FCC 4*64^3, side (N/0.83134)^0.3333333, list cutoff 3.5*1.2 periodic
    -> 130,023,424 (moldyn/moldyn.h:20, moldyn/irresult/2:5)."""
    O = oracle_lib
    n = 4 * 64 ** 3
    side = (n / 0.83134) ** 0.3333333
    assert abs(side - 108.045548) < 1e-5
    pos = O.fcc_moldyn(64, side).astype(np.float32)
    assert O.neighbor_count(pos, float(np.float32(side)), np.float32((3.5 * 1.2) ** 2)) == 130023424


def test_partition_oracle_properties(oracle_lib):
    O = oracle_lib
    c = load_golden("moldyn_shuffled_dups_1500")
    pos32 = c["pos"].astype(np.float32)
    lo, scale = O.morton_frame(pos32)
    perm, inv, row_off, col = O.partition(pos32, lo, scale, c["edges"])
    n = pos32.shape[0]
    assert np.array_equal(np.sort(perm), np.arange(n))
    assert np.array_equal(inv[perm], np.arange(n))
    keys = O.morton_keys(pos32, lo, scale)
    ks = keys[perm]
    assert np.all(ks[:-1] <= ks[1:])
    # stability: equal keys keep node order
    same = ks[:-1] == ks[1:]
    assert np.all(perm[:-1][same] < perm[1:][same])
    # rows hold exactly each node's incident edges
    e = c["edges"]
    deg = np.bincount(inv[e[:, 0]], minlength=n) + np.bincount(inv[e[:, 1]], minlength=n)
    assert np.array_equal(np.diff(row_off), deg)
    assert row_off[-1] == 2 * e.shape[0]
    # entry order within a row: columns ascending (duplicate edges adjacent)
    r = int(np.argmax(deg))
    seq = []
    for t, (a, b) in enumerate(e):
        if inv[a] == r:
            seq.append(inv[b])
        if inv[b] == r:
            seq.append(inv[a])
    assert np.array_equal(col[row_off[r]:row_off[r + 1]], np.sort(np.array(seq, np.int32)))
    for q in range(n):
        assert np.all(np.diff(col[row_off[q]:row_off[q + 1]]) >= 0)
    # the layout does not depend on the order of the edge list
    rng = np.random.default_rng(5)
    shuf = e[rng.permutation(e.shape[0])].copy()
    flip = rng.random(e.shape[0]) < 0.5
    shuf[flip] = shuf[flip][:, ::-1]
    _, _, row_off2, col2 = O.partition(pos32, lo, scale, shuf)
    assert np.array_equal(row_off2, row_off) and np.array_equal(col2, col)


def test_hilbert_keys_walk_the_grid(oracle_lib):
    """The partition's Hilbert key: the first 8^4 keys fill the 16^3 corner
    cube, each key's cell is face-adjacent to the next one's, and distinct
    cells get distinct keys."""
    O = oracle_lib
    g = np.arange(16, dtype=np.float32)
    cells = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3) + np.float32(0.5)
    lo = np.zeros(3, np.float32)
    scale = np.ones(3, np.float32)  # quantisation: cell (i, j, k) -> (i, j, k)
    keys = O.hilbert_keys(cells, lo, scale)
    assert np.array_equal(np.sort(keys), np.arange(16 ** 3, dtype=np.uint32))
    path = cells[np.argsort(keys)]
    assert np.all(np.abs(np.diff(path, axis=0)).sum(axis=1) == 1)
    rng = np.random.default_rng(3)
    far = rng.integers(0, 1024, size=(1024, 3)).astype(np.float32) + np.float32(0.5)
    far = np.unique(far, axis=0)
    assert np.unique(O.hilbert_keys(far, lo, scale)).size == far.shape[0]

