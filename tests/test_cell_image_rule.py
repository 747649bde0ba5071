"""The neighbour search's cell-decided periodic image, checked on the CPU.

The pair rule wraps each float difference d = a - b once by +-box when
|d| > box/2.  With at least 5 cells per axis and positions in [0, box), the
search instead adds the shift of the neighbour cell (0, or +-box for a cell
reached across the boundary).  Per axis the two must give the same d up to the
sign of zero (d enters only squared), for every pair of positions in the same
or adjacent cells -- including positions on and next to the cell boundaries,
0, -0 and the last float below the box.  Cells are assigned as the search
assigns them: floor(x * (1 / (box / nc))) in double, wrapped and clamped.
"""
import numpy as np
import pytest


def cells_of(x, box, nc):
    csz = float(box) / nc
    k = np.floor(x.astype(np.float64) * (1.0 / csz)).astype(np.int64)
    k = ((k % nc) + nc) % nc
    return np.clip(k, 0, nc - 1)


def axis_positions(box, nc, rng, count=3000):
    box = np.float32(box)
    x = (rng.random(count, dtype=np.float32) * box).astype(np.float32)
    special = [np.float32(0.0), np.float32(-0.0), np.nextafter(box, np.float32(0))]
    for b in (box / np.float32(nc)) * np.arange(1, nc, dtype=np.float32):
        special += [b, np.nextafter(b, np.float32(0)), np.nextafter(b, box)]
    x = np.concatenate([x, np.array(special, np.float32)])
    return x[(x >= 0) & (x < box)]


def rule(a, b, box):
    hb = np.float32(0.5) * box
    d = (a - b).astype(np.float32)
    d = np.where(d > hb, (d - box).astype(np.float32), d)
    d = np.where(d < -hb, (d + box).astype(np.float32), d)
    return d


def mismatches(box, nc, seed):
    box = np.float32(box)
    rng = np.random.Generator(np.random.PCG64(seed))
    x = axis_positions(box, nc, rng)
    k = cells_of(x, box, nc)
    a, b = np.meshgrid(x, x, indexing="ij")
    ka, kb = np.meshgrid(k, k, indexing="ij")
    step = (kb - ka) % nc
    near = (step == 0) | (step == 1) | (step == nc - 1)
    # the neighbour cell's shift: reached below 0 (ka = 0, kb = nc - 1) -> +box,
    # past the top (ka = nc - 1, kb = 0) -> -box
    s = np.where((ka == 0) & (kb == nc - 1), box, np.where((ka == nc - 1) & (kb == 0), -box, np.float32(0)))
    s = s.astype(np.float32)
    shifted = ((a - b).astype(np.float32) + s).astype(np.float32)
    want = rule(a, b, box)
    bad = near & (shifted * shifted != want * want)
    return int(bad.sum()), int(near.sum())


@pytest.mark.parametrize("nc", [5, 6, 7, 12, 38])
@pytest.mark.parametrize("box", [13.5, 19.226577758789062, 107.4, 170.7])
def test_cell_shift_equals_the_rule(box, nc):
    bad, pairs = mismatches(box, nc, seed=nc * 1000 + int(box))
    assert pairs > 100_000
    assert bad == 0


def test_three_cells_are_not_enough():
    """At 3 cells per axis two adjacent cells reach 2/3 of the box: the rule
    wraps pairs the cells call unwrapped, so the search keeps the per-pair
    test there (it takes the cell-decided image from 5 cells up)."""
    bad, _ = mismatches(19.226577758789062, 3, seed=3)
    assert bad > 0
