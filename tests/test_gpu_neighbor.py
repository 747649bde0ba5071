"""The GPU neighbour-list builder (irr_neighbor_build) against the oracle (GPU).

The half list (i < j, sorted by i then j) is integer output: it must equal the
oracle's list bit for bit, and reproduce the two list sizes the reference
logs (miniMD 18,816,288; moldyn 130,023,424).
"""
import numpy as np
import pytest

from helpers import TOL_PERNODE_F64, random_box, scaled_error

pytestmark = pytest.mark.gpu


def gpu_list(irr, pos32, box, cut2):
    d = irr.neighbor_build(pos32, float(box), float(cut2))
    try:
        return d.to_host()
    finally:
        d.close()


@pytest.mark.parametrize("case", ["periodic_random", "open_fcc", "tiny_periodic_box",
                                  "dense_cluster"])
def test_list_equals_oracle(built_lib, oracle_lib, case):
    import irregular_gb300 as irr
    O = oracle_lib
    rng = np.random.Generator(np.random.PCG64(99))
    if case == "periodic_random":
        pos32, L = random_box(20000, 0.9, 31)
        box, cut2 = float(L), np.float32(2.5 * 2.5)
    elif case == "open_fcc":
        pos32 = O.fcc_minimd(12, 12, 12, 0.8442).astype(np.float32)
        pos32 = (pos32 + rng.normal(0, 0.04, pos32.shape).astype(np.float32)).astype(np.float32)
        box, cut2 = 0.0, np.float32(2.8 * 2.8)
    elif case == "tiny_periodic_box":   # fewer than 3 cells per side: deduplicated offsets
        L = np.float32(5.0)
        pos32 = (rng.random((300, 3), dtype=np.float32) * L).astype(np.float32)
        pos32[pos32 >= L] = 0
        box, cut2 = float(L), np.float32(2.0 * 2.0)
    else:  # 1,500 nodes inside one cutoff sphere: rows longer than the shared row sort holds
        L = np.float32(40.0)
        bulk = (rng.random((4000, 3), dtype=np.float32) * L).astype(np.float32)
        blob = (np.float32(20.0) + rng.random((1500, 3), dtype=np.float32)).astype(np.float32)
        pos32 = np.concatenate([bulk, blob]).astype(np.float32)
        pos32[pos32 >= L] = 0
        box, cut2 = float(L), np.float32(2.5 * 2.5)
    got = gpu_list(irr, pos32, box, cut2)
    ref = O.neighbor_half_list(pos32, box, cut2)
    assert np.array_equal(got, ref)
    if case == "dense_cluster":
        assert np.bincount(got[:, 0]).max() > 1024


def boundary_box(seed: int, outside: bool):
    """6,000 nodes, 7 cells per axis at cutoff 2.5 (the builder then takes each
    pair's periodic image from its cell): a tenth of the coordinates moved onto
    the places where that matters -- 0, -0, the last float below the box, each
    cell boundary and its neighbouring floats.  With outside, some nodes also
    sit up to 0.3 outside [0, box) or exactly on the box, where the builder
    goes back to the per-pair rule."""
    pos32, L = random_box(6000, 0.8442, seed)
    assert int(np.floor(float(L) / (2.5 * 1.0001 + 1e-12))) == 7
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    edges = np.float32(L) / np.float32(7) * np.arange(8, dtype=np.float32)
    special = [np.float32(0.0), np.float32(-0.0), np.nextafter(np.float32(L), np.float32(0))]
    for b in edges[1:7]:
        special += [b, np.nextafter(b, np.float32(0)), np.nextafter(b, np.float32(L))]
    if outside:
        special += [np.float32(-0.3), np.float32(-0.2), np.float32(L),
                    np.float32(L + np.float32(0.2)), np.float32(L + np.float32(0.3))]
    k = rng.integers(0, pos32.size, size=pos32.size // 10)
    flat = pos32.reshape(-1)
    flat[k] = np.array(special, np.float32)[rng.integers(0, len(special), size=k.size)]
    return pos32, float(L)


@pytest.mark.parametrize("outside", [False, True])
def test_cell_decided_image_at_the_boundaries(built_lib, oracle_lib, outside):
    import irregular_gb300 as irr
    pos32, L = boundary_box(7, outside)
    cut2 = np.float32(2.5 * 2.5)
    ref = oracle_lib.neighbor_half_list(pos32, L, cut2)
    assert np.array_equal(gpu_list(irr, pos32, L, cut2), ref)
    if outside:
        return
    # the MD loop's half-stencil build (each pair found once, from one end):
    # its list size and the forces over it (law cutoff 2.2, list 2.2 + 0.3)
    md = irr.MD(pos32.astype(np.float64), np.zeros((pos32.shape[0], 3)), L, cutforce=2.2, skin=0.3)
    try:
        assert md.info().num_edges == ref.shape[0]
        f = md.forces()
    finally:
        md.close()
    f64, sabs = oracle_lib.lj_reduce_f64(pos32.astype(np.float64), ref,
                                         oracle_lib.lj_param(2.2 ** 2, L, True))
    # per node, against the sum of its terms' magnitudes (a close pair's huge
    # force would make a norm-wise bound meaningless for the rest)
    assert scaled_error(f, 48.0 * f64, 48.0 * sabs) <= TOL_PERNODE_F64


def test_known_answer_minimd(built_lib, oracle_lib):
    """miniMD lj.in: FCC 50^3 at rho 0.8442, cutneigh 2.8, open box (miniMD/2:13)."""
    import irregular_gb300 as irr
    O = oracle_lib
    pos32 = O.fcc_minimd(50, 50, 50, 0.8442).astype(np.float32)
    assert pos32.shape[0] == 500000
    d = irr.neighbor_build(pos32, 0.0, 2.8 * 2.8)
    assert d.count == 18816288
    d.close()


def test_known_answer_minimd_periodic(built_lib, oracle_lib):
    """The same lattice with periodic images: every atom has the 78 lattice
    neighbours of the first five FCC shells inside 2.8 (the sixth is at
    2.91), so the half list holds 39 per atom: 19,500,000."""
    import irregular_gb300 as irr
    O = oracle_lib
    pos32 = O.fcc_minimd(50, 50, 50, 0.8442).astype(np.float32)
    side = float(np.float32(50 * (4 / 0.8442) ** (1 / 3)))
    d = irr.neighbor_build(pos32, side, 2.8 * 2.8)
    assert d.count == 19500000
    d.close()


def test_known_answer_moldyn(built_lib, oracle_lib):
    """moldyn: FCC 4*64^3, side (N/0.83134)^0.3333333, list cutoff 3.5*1.2,
    periodic (moldyn/moldyn.h:20, moldyn/irresult/2:5)."""
    import irregular_gb300 as irr
    O = oracle_lib
    side = (4 * 64 ** 3 / 0.83134) ** 0.3333333
    assert abs(side - 108.045548) < 1e-5
    pos32 = O.fcc_moldyn(64, side).astype(np.float32)
    d = irr.neighbor_build(pos32, float(np.float32(side)), float(np.float32((3.5 * 1.2) ** 2)))
    assert d.count == 130023424
    d.close()
