"""The allocation-free Morton ordering (irr_morton_order_static), through the C ABI (GPU).

Some callers cannot allocate device memory -- an application that reserved
the GPU's memory for its own pool, or a latency-bound loop that must not pay
for cudaMalloc/cudaFree.  For them the library offers one entry point whose
scratch is a fixed device array inside the library.  Its output must be the
node permutation the partitioner itself produces (integers: bit for bit), on
two calls in a row, since the calls share that array.

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import numpy as np
import pytest

from helpers import random_box

pytestmark = pytest.mark.gpu


def partitioner_perm(irr, pos32):
    """The existing path: a partitioned handle's Morton permutation."""
    h = irr.Handle(irr.default_config(map_idx=irr.IRR_MAP_LJ_MOLDYN, exec=irr.IRR_EXEC_PARTITIONED,
                                      reorder=1, order=irr.IRR_ORDER_MORTON))
    h.set_params(irr.moldyn_params(1000.0, 2.5))
    h.set_edges(np.zeros((0, 2), np.int32))
    h.set_nodes(pos32, 12)
    h.init()
    perm, _, _ = h.partition()
    h.close()
    return perm


def static_perm(irr, torch, d_pos, elm, n):
    out = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    rc = irr.load().irr_morton_order_static(0, None, d_pos.data_ptr(), elm, n, out.data_ptr())
    assert rc == irr.IRR_OK, irr.load().irr_status_string(rc)
    torch.cuda.synchronize()
    return out[:n].cpu().numpy()


@pytest.mark.parametrize("n,seed", [(1, 1), (2, 2), (5000, 3), (65536, 4), (1048576, 5)])
def test_static_ordering_matches_partitioner_twice(built_lib, n, seed):
    torch = pytest.importorskip("torch")
    import irregular_gb300 as irr
    pos32, _ = random_box(n, 0.9, seed)
    ref = partitioner_perm(irr, pos32)
    d12 = torch.from_numpy(pos32).cuda()
    d16 = torch.from_numpy(np.concatenate([pos32, np.ones((n, 1), np.float32)], 1)).cuda()
    first = static_perm(irr, torch, d12, 12, n)
    second = static_perm(irr, torch, d16, 16, n)
    assert np.array_equal(first, ref)
    assert np.array_equal(second, ref)


def test_static_ordering_after_a_different_size(built_lib):
    """The shared array keeps the previous call's contents; a smaller call after a
    larger one must not see them."""
    torch = pytest.importorskip("torch")
    import irregular_gb300 as irr
    big, _ = random_box(300000, 0.9, 11)
    small, _ = random_box(777, 0.9, 12)
    static_perm(irr, torch, torch.from_numpy(big).cuda(), 12, big.shape[0])
    got = static_perm(irr, torch, torch.from_numpy(small).cuda(), 12, small.shape[0])
    assert np.array_equal(got, partitioner_perm(irr, small))


@pytest.mark.parametrize("case", ["flat_axis", "signed_zero_minimum"])
def test_static_ordering_degenerate_frames(built_lib, case):
    """Where the two routes form the curve frame differently (on the device here,
    on the host after a warp reduction in the partitioner): an axis with no
    extent (scale 0), and an axis whose minimum is +0.0 for some nodes and -0.0
    for others."""
    torch = pytest.importorskip("torch")
    import irregular_gb300 as irr
    pos32, _ = random_box(20000, 0.9, 21)
    if case == "flat_axis":
        pos32[:, 2] = np.float32(1.5)
    else:
        pos32[::3, 0] = np.float32(0.0)
        pos32[1::3, 0] = np.float32(-0.0)
    ref = partitioner_perm(irr, pos32)
    got = static_perm(irr, torch, torch.from_numpy(pos32).cuda(), 12, pos32.shape[0])
    again = static_perm(irr, torch, torch.from_numpy(pos32).cuda(), 12, pos32.shape[0])
    assert np.array_equal(got, ref)
    assert np.array_equal(again, ref)


def test_static_ordering_rejects_oversize_and_bad_args(built_lib):
    torch = pytest.importorskip("torch")
    import irregular_gb300 as irr
    L = irr.load()
    d = torch.zeros(16, dtype=torch.float32, device="cuda")
    o = torch.zeros(4, dtype=torch.int32, device="cuda")
    assert L.irr_morton_order_static(0, None, d.data_ptr(), 12, 1048577, o.data_ptr()) == \
        irr.IRR_ERR_CAPACITY
    assert L.irr_morton_order_static(0, None, d.data_ptr(), 24, 4, o.data_ptr()) == irr.IRR_ERR_ARG
    assert L.irr_morton_order_static(0, None, None, 12, 4, o.data_ptr()) == irr.IRR_ERR_ARG
    assert L.irr_morton_order_static(0, None, d.data_ptr(), 12, 0, None) == irr.IRR_OK
    # records and output are read and written as 4-byte words
    assert L.irr_morton_order_static(0, None, d.data_ptr() + 2, 12, 4, o.data_ptr()) == \
        irr.IRR_ERR_ARG
    assert L.irr_morton_order_static(0, None, d.data_ptr(), 12, 2, o.data_ptr() + 1) == \
        irr.IRR_ERR_ARG
