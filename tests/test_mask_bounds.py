"""The per-row step bounds that replace the per-step entry masks in the
partitioned kernels' loops (csrc/irr_reduce.cu: consume_halo, consume_sliced).

A row of `len` entries is walked by G lanes, two entries per lane per step:
lane l takes entry 2G t + l and entry 2G t + l + G at step t.  The kernels
compute, once per row,

    n0 = ceil((len - l) / 2G)       if len > l       else 0
    n1 = ceil((len - l - G) / 2G)   if len > l + G   else 0

and test t < n0, t < n1 (as bounds on the step's shared address) instead of
the two index comparisons per step.  This checks the equivalence for every
row length the layouts allow, on the CPU."""
import numpy as np
import pytest


def bounds(length, lane, G):
    n0 = (length - lane + 2 * G - 1) // (2 * G) if length > lane else 0
    n1 = (length - lane - G + 2 * G - 1) // (2 * G) if length > lane + G else 0
    return n0, n1


@pytest.mark.parametrize("G", [1, 2, 4, 8, 16, 32])
def test_bounds_equal_the_index_masks(G):
    lens = np.arange(0, 1024 if G == 4 else 600)
    for lane in range(G):
        steps = (lens.max() + 2 * G - 1) // (2 * G) + 2
        t = np.arange(steps)[None, :]
        want0 = 2 * G * t + lane < lens[:, None]
        want1 = 2 * G * t + lane + G < lens[:, None]
        nb = np.array([bounds(int(n), lane, G) for n in lens])
        assert np.array_equal(t < nb[:, :1], want0), (G, lane)
        assert np.array_equal(t < nb[:, 1:], want1), (G, lane)


def test_staged_address_form():
    """consume_halo: step t reads its word at base + 128 (t + 1) after the
    increment, and tests addr <= base + 128 n; the same as t < n."""
    base = 0x1234 * 4
    for length in range(0, 1024):
        for lane in range(4):
            n0, n1 = bounds(length, lane, 4)
            steps = (length + 7) // 8 + 1
            for t in range(steps):
                addr = base + 128 * (t + 1)
                assert (addr <= base + 128 * n0) == (8 * t + lane < length)
                assert (addr <= base + 128 * n1) == (8 * t + lane + 4 < length)
