"""Parity of the CUDA reduction with the oracle, through the C ABI (GPU).

Every case compares the GPU result with
  * the reference's own CPU result (golden fixtures): per node and component
    within 1e-5 of the FP64 absolute-term scale (FP32 reordering), and
  * the FP64 oracle: normwise max|df|/max|f| <= 1e-6.
Integer outputs (the partition) are compared bit for bit.
"""
import numpy as np
import pytest

from helpers import (TOL_NORMWISE_F64, TOL_PERNODE_F64, TOL_VS_REFERENCE, golden_names,
                     load_golden, map_idx_of, normwise_error, oracle_param, random_box,
                     scaled_error)

pytestmark = pytest.mark.gpu

SHAPES = {
    "plain": dict(exec=0),
    "part": dict(exec=1),
    "part_g1": dict(exec=1, lanes_per_row=1),
    "part_g2": dict(exec=1, lanes_per_row=2),
    "part_g4": dict(exec=1, lanes_per_row=4),
    "part_g16": dict(exec=1, lanes_per_row=16),
    "part_g32": dict(exec=1, lanes_per_row=32),
    "part_direct": dict(exec=1, stage_smem=0),
    "part_b2048": dict(exec=1, block_nodes=2048),
    "part_b64": dict(exec=1, block_nodes=64),
    "part_noreorder": dict(exec=1, reorder=0),
    "csr": dict(exec=1, layout=1),
    "sliced": dict(exec=1, layout=2),
    "sliced_g1": dict(exec=1, layout=2, lanes_per_row=1),
    "sliced_g2": dict(exec=1, layout=2, lanes_per_row=2),
    "sliced_g8": dict(exec=1, layout=2, lanes_per_row=8),
    "sliced_g16": dict(exec=1, layout=2, lanes_per_row=16),
    "sliced_g32": dict(exec=1, layout=2, lanes_per_row=32),
    "sliced_direct": dict(exec=1, layout=2, stage_smem=0),
    "sliced_b64": dict(exec=1, layout=2, block_nodes=64),
    "sliced_noreorder": dict(exec=1, layout=2, reorder=0),
}


def run_case(irr, case, elm_out=12, **cfg):
    h = irr.Handle(irr.default_config(map_idx=map_idx_of(case), **cfg))
    h.set_params(case["param"])
    h.set_edges(case["edges"])
    h.set_nodes(case["pos"], 24)
    h.step()
    f = h.get_result(elm_size=elm_out)
    return f, h


@pytest.mark.parametrize("shape", sorted(SHAPES))
@pytest.mark.parametrize("name", golden_names())
def test_parity_golden(built_lib, oracle_lib, name, shape):
    import irregular_gb300 as irr
    O = oracle_lib
    c = load_golden(name)
    f, h = run_case(irr, c, **SHAPES[shape])
    f64, sabs = O.lj_reduce_f64(c["pos"], c["edges"], oracle_param(O, c))
    assert scaled_error(f, c["f_ref"], sabs) <= TOL_VS_REFERENCE
    assert normwise_error(f, f64) <= TOL_NORMWISE_F64
    assert scaled_error(f, f64, sabs) <= TOL_PERNODE_F64
    h.close()


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("reorder,curve", [(1, "hilbert"), (1, "morton"), (0, "morton")])
def test_partition_bit_exact(built_lib, oracle_lib, name, reorder, curve):
    import irregular_gb300 as irr
    O = oracle_lib
    c = load_golden(name)
    order = irr.IRR_ORDER_HILBERT if curve == "hilbert" else irr.IRR_ORDER_MORTON
    h = irr.Handle(irr.default_config(map_idx=map_idx_of(c), exec=1, reorder=reorder, order=order))
    h.set_params(c["param"])
    h.set_edges(c["edges"])
    h.set_nodes(c["pos"], 24)
    h.init()
    perm, row_off, col = h.partition()
    pos32 = c["pos"].astype(np.float32)
    if reorder:
        lo, scale = O.morton_frame(pos32)
    else:
        lo, scale = np.zeros(3, np.float32), np.zeros(3, np.float32)  # all keys 0: identity
    operm, oinv, orow, ocol = O.partition(pos32, lo, scale, c["edges"], curve=curve)
    assert h.info().order == order
    assert np.array_equal(perm, operm)
    assert np.array_equal(row_off, orow)
    assert np.array_equal(col, ocol)


def test_partition_rows_of_every_sort_path_bit_exact(built_lib, oracle_lib):
    """Rows of 1..~1000 entries (with duplicate edges) take every row-sort path
    -- 1, 2, 4 and 8 entries per lane in registers, and shared memory above
    256 -- and still equal the oracle's partition bit for bit."""
    import irregular_gb300 as irr
    O = oracle_lib
    rng = np.random.default_rng(77)
    n = 3000
    pos32, L = random_box(n, 0.8442, 78)
    edges = [rng.integers(0, n, size=(6000, 2))]
    for k, d in enumerate([1, 2, 31, 33, 64, 65, 127, 129, 200, 256, 257, 400, 700, 900]):
        hub = 17 * k + 5
        others = rng.choice(np.delete(np.arange(n), hub), size=d, replace=False)
        edges.append(np.stack([np.full(d, hub), others], axis=1))
    e = np.concatenate(edges).astype(np.int32)
    e = e[e[:, 0] != e[:, 1]]
    e = np.concatenate([e, e[rng.choice(e.shape[0], 500)]])  # duplicates
    e = e[rng.permutation(e.shape[0])]
    h = irr.Handle(irr.default_config(map_idx=0, exec=1))
    h.set_params(irr.moldyn_params(float(L), 2.5))
    h.set_edges(e)
    h.set_nodes(pos32, 12)
    h.init()
    perm, row_off, col = h.partition()
    deg = np.diff(row_off.astype(np.int64))
    assert deg.max() <= 1024 and (deg > 256).sum() >= 3 and ((deg > 128) & (deg <= 256)).sum() >= 3
    lo, scale = O.morton_frame(pos32)
    operm, _, orow, ocol = O.partition(pos32, lo, scale, e, curve="hilbert")
    assert np.array_equal(perm, operm)
    assert np.array_equal(row_off, orow)
    assert np.array_equal(col, ocol)
    h.close()


@pytest.mark.parametrize("shape", ["part", "part_direct", "part_g32", "part_g1"])
def test_partitioned_is_bitwise_reproducible(built_lib, shape):
    import irregular_gb300 as irr
    c = load_golden("moldyn_random_2048")
    f1, h1 = run_case(irr, c, **SHAPES[shape])
    h1.step()
    f2 = h1.get_result(elm_size=12)
    f3, _ = run_case(irr, c, **SHAPES[shape])
    assert np.array_equal(f1.view(np.uint32), f2.view(np.uint32))
    assert np.array_equal(f1.view(np.uint32), f3.view(np.uint32))


@pytest.mark.parametrize("shape", ["part", "part_g1", "part_noreorder"])
def test_partitioned_result_ignores_edge_order(built_lib, shape):
    """Rows are laid out in (row, col) order, so a shuffled edge list with
    flipped endpoints gives the same bits."""
    import irregular_gb300 as irr
    c = dict(load_golden("moldyn_shuffled_dups_1500"))
    f1, _ = run_case(irr, c, **SHAPES[shape])
    rng = np.random.default_rng(11)
    e = c["edges"][rng.permutation(c["edges"].shape[0])].copy()
    flip = rng.random(e.shape[0]) < 0.5
    e[flip] = e[flip][:, ::-1]
    c["edges"] = e
    f2, _ = run_case(irr, c, **SHAPES[shape])
    assert np.array_equal(f1.view(np.uint32), f2.view(np.uint32))


@pytest.mark.parametrize("lanes", [1, 2, 4, 8, 16, 32])
@pytest.mark.parametrize("name", golden_names())
def test_sliced_layout_gives_the_csr_sums(built_lib, name, lanes):
    """The sliced layout hands every lane the entry pairs CSR gives it, in the
    same order, so the sums agree exactly."""
    import irregular_gb300 as irr
    c = load_golden(name)
    f_csr, h1 = run_case(irr, c, exec=1, layout=irr.IRR_LAYOUT_CSR, lanes_per_row=lanes)
    f_sl, h2 = run_case(irr, c, exec=1, layout=irr.IRR_LAYOUT_SLICED, lanes_per_row=lanes)
    f_dir, h3 = run_case(irr, c, exec=1, layout=irr.IRR_LAYOUT_SLICED, lanes_per_row=lanes,
                         stage_smem=0)
    assert h1.info().layout == irr.IRR_LAYOUT_CSR and h2.info().layout == irr.IRR_LAYOUT_SLICED
    assert np.array_equal(f_csr, f_sl) and np.array_equal(f_csr, f_dir)
    inf = h2.info()
    assert inf.num_slots >= inf.num_entries and inf.num_slots % 64 == 0


def test_auto_layout_choice(built_lib):
    """AUTO takes the staged layout where it applies (4 lanes per row, the
    shared-memory stages, tables within their limit), else the sliced layout
    for near-uniform rows, and keeps CSR when long rows would make the padding
    dominate."""
    import irregular_gb300 as irr
    c = load_golden("moldyn_random_2048")
    _, h = run_case(irr, c, exec=1)
    assert h.info().layout == irr.IRR_LAYOUT_STAGED
    for cfg in (dict(lanes_per_row=8), dict(stage_smem=0)):
        _, hs = run_case(irr, c, exec=1, **cfg)
        assert hs.info().layout == irr.IRR_LAYOUT_SLICED, cfg
        hs.close()
    n = c["pos"].shape[0]
    # 32 hub nodes joined to every other node: their slices pad 8 rows each
    # to ~n entries, far more than half the entries
    hubs = [np.stack([np.full(n - 1, k, np.int32), np.delete(np.arange(n, dtype=np.int32), k)],
                     axis=1) for k in range(0, n, n // 32)]
    skew = dict(c)
    skew["edges"] = np.concatenate([c["edges"]] + hubs).astype(np.int32)
    f, h2 = run_case(irr, skew, exec=1)
    assert h2.info().layout == irr.IRR_LAYOUT_CSR
    f_sl, h3 = run_case(irr, skew, exec=1, layout=irr.IRR_LAYOUT_SLICED)
    assert h3.info().layout == irr.IRR_LAYOUT_SLICED
    assert np.array_equal(f, f_sl)


@pytest.mark.parametrize("exec_mode", [0, 1])
def test_result_formats_agree(built_lib, exec_mode):
    import irregular_gb300 as irr
    c = load_golden("minimd_fcc_864")
    f12, h = run_case(irr, c, exec=exec_mode)
    f16 = h.get_result(elm_size=16)
    f24 = h.get_result(elm_size=24)
    assert np.array_equal(f12, f16[:, :3]) and np.all(f16[:, 3] == 0)
    assert np.array_equal(f12.astype(np.float64), f24)


@pytest.mark.parametrize("offset", [0, 4])
@pytest.mark.parametrize("exec_mode", [0, 1])
@pytest.mark.parametrize("fmt", [12, 16, 24])
def test_page_locked_host_buffers(built_lib, exec_mode, fmt, offset):
    """Page-locked caller buffers on a 16-byte boundary are read and written
    by the kernels in place; other buffers (offset 4) go through staging.
    Either way the partitioned results equal those through pageable buffers
    bit for bit (the plain path's atomics only to rounding)."""
    torch = pytest.importorskip("torch")
    import irregular_gb300 as irr
    c = load_golden("moldyn_random_2048")
    n = c["pos"].shape[0]
    dt = np.float64 if fmt == 24 else np.float32
    width = fmt // np.dtype(dt).itemsize
    rec = np.zeros((n, width), dt)
    rec[:, :3] = c["pos"]
    moved = rec.copy()
    moved[:, :3] += np.random.Generator(np.random.PCG64(3)).normal(0, 1e-3, (n, 3)).astype(dt)
    h = irr.Handle(irr.default_config(map_idx=0, exec=exec_mode))
    h.set_params(c["param"])
    h.set_edges(c["edges"])
    h.set_nodes(rec, fmt)
    h.step()
    h.set_nodes(moved, fmt)  # pageable: staged
    h.step()
    ref = h.get_result(elm_size=fmt)

    def pinned_view(shape, dtype):
        raw = torch.empty(int(np.prod(shape)) * np.dtype(dtype).itemsize + 16, dtype=torch.uint8,
                          pin_memory=True).numpy()
        return np.frombuffer(raw.data, dtype=dtype, count=int(np.prod(shape)),
                             offset=offset).reshape(shape), raw

    h.set_nodes(rec, fmt)
    h.step()
    view_in, keep_in = pinned_view(moved.shape, dt)
    view_in[:] = moved
    h.set_nodes(view_in, fmt)
    h.step()
    view_out, keep_out = pinned_view(ref.shape, ref.dtype)
    h.get_result(view_out, elm_size=fmt)
    if exec_mode == 1:
        assert np.array_equal(view_out.view(np.uint8), ref.view(np.uint8))
    else:  # the plain path's float atomics add in no fixed order
        assert normwise_error(view_out[:, :3], ref[:, :3]) <= TOL_NORMWISE_F64
    h.close()


def test_device_result_buffer_alignment_is_checked(built_lib):
    torch = pytest.importorskip("torch")
    import irregular_gb300 as irr
    c = load_golden("moldyn_random_2048")
    f, h = run_case(irr, c, exec=1)
    d = torch.zeros(c["pos"].shape[0] * 6 + 4, dtype=torch.float32, device="cuda")
    with pytest.raises(irr.IrregularError) as ei:
        h.get_result_device(d[1:], elm_size=24)  # 4-byte aligned, 8 needed
    assert ei.value.status == irr.IRR_ERR_ARG
    h.get_result_device(d[2:], elm_size=24)
    torch.cuda.synchronize()
    got = d[2:2 + 6 * f.shape[0]].cpu().numpy().view(np.float64).reshape(-1, 3)
    assert np.array_equal(got, f.astype(np.float64))
    h.close()


@pytest.mark.parametrize("exec_mode", [0, 1])
@pytest.mark.parametrize("fmt", [12, 16, 24])
def test_reset_node_data(built_lib, oracle_lib, exec_mode, fmt):
    """reset_node_data between iterations (irregular_runtime.cu:436-439), every node format."""
    import irregular_gb300 as irr
    O = oracle_lib
    c = load_golden("moldyn_random_2048")
    h = irr.Handle(irr.default_config(map_idx=0, exec=exec_mode))
    h.set_params(c["param"])
    h.set_edges(c["edges"])
    h.set_nodes(c["pos"], 24)
    h.step()
    rng = np.random.Generator(np.random.PCG64(11))
    L = np.float32(c["side"])
    pos2 = ((c["pos"].astype(np.float32) + rng.normal(0, 0.05, c["pos"].shape).astype(np.float32))
            % L).astype(np.float32)
    if fmt == 24:
        h.set_nodes(pos2.astype(np.float64), 24)
    elif fmt == 16:
        h.set_nodes(np.concatenate([pos2, np.full((pos2.shape[0], 1), 7, np.float32)], 1), 16)
    else:
        h.set_nodes(pos2, 12)
    h.step()
    f = h.get_result(elm_size=12)
    p = oracle_param(O, c)
    f64, sabs = O.lj_reduce_f64(pos2.astype(np.float64), c["edges"], p)
    fr = O.lj_reduce_refnum(pos2.astype(np.float64), c["edges"], p)
    assert scaled_error(f, fr, sabs) <= TOL_VS_REFERENCE
    assert normwise_error(f, f64) <= TOL_NORMWISE_F64


@pytest.mark.parametrize("exec_mode", [0, 1])
def test_empty_edge_list(built_lib, exec_mode):
    import irregular_gb300 as irr
    h = irr.Handle(irr.default_config(map_idx=0, exec=exec_mode))
    h.set_params(irr.moldyn_params(20.0, 2.5))
    h.set_edges(np.zeros((0, 2), np.int32))
    h.set_nodes(np.random.default_rng(0).random((100, 3)) * 20, 24)
    h.step()
    assert np.all(h.get_result(elm_size=12) == 0)


@pytest.mark.parametrize("exec_mode", [0, 1])
def test_out_of_range_endpoint_is_an_error(built_lib, exec_mode):
    import irregular_gb300 as irr
    h = irr.Handle(irr.default_config(map_idx=0, exec=exec_mode))
    h.set_params(irr.moldyn_params(20.0, 2.5))
    h.set_edges(np.array([[0, 1], [2, 100]], np.int32))
    h.set_nodes(np.random.default_rng(0).random((100, 3)) * 20, 24)
    with pytest.raises(irr.IrregularError) as ei:
        h.step()
    assert ei.value.status == irr.IRR_ERR_INDEX
    h.set_edges(np.array([[0, 1], [-1, 3]], np.int32))
    with pytest.raises(irr.IrregularError) as ei:
        h.init()
    assert ei.value.status == irr.IRR_ERR_INDEX


@pytest.mark.parametrize("exec_mode", [0, 1])
def test_self_loop_gives_nan_like_reference(built_lib, oracle_lib, exec_mode):
    """An edge (i, i) has rd = 0 < cutoff^2: the reference's map computes
    inf - inf and inserts NaN; so does the kernel.  Other nodes are unaffected."""
    import irregular_gb300 as irr
    O = oracle_lib
    pos = np.array([[1, 1, 1], [2, 1, 1], [5, 5, 5], [5.5, 5, 5]], np.float64)
    edges = np.array([[0, 1], [2, 2], [2, 3]], np.int32)
    h = irr.Handle(irr.default_config(map_idx=0, exec=exec_mode))
    h.set_params(irr.moldyn_params(20.0, 2.5))
    h.set_edges(edges)
    h.set_nodes(pos, 24)
    h.step()
    f = h.get_result(elm_size=12)
    fr = O.lj_reduce_refnum(pos, edges, O.lj_param(6.25, 20.0, True))
    assert np.array_equal(np.isnan(f), np.isnan(fr))
    assert np.all(np.isnan(f[2])) and not np.any(np.isnan(f[[0, 1]]))
    assert np.allclose(f[[0, 1]], fr[[0, 1]], rtol=1e-6)


def test_cutoff_boundary_follows_reference_decision(built_lib, oracle_lib):
    """Pairs within a few ulps of the cutoff take the reference's FP64 decision."""
    import irregular_gb300 as irr
    O = oracle_lib
    rc = 2.5
    # distances straddling rc by a few float ulps along x
    base = np.float32(10.0)
    xs = [np.nextafter(np.float32(base + rc), np.float32(k), dtype=np.float32) for k in (0, 100)]
    xs += [np.float32(base + rc)]
    pos = [[base, 5, 5]]
    for x in xs:
        pos.append([x, 5, 5])
    pos = np.array(pos, np.float32).astype(np.float64)
    edges = np.array([[0, k] for k in range(1, len(pos))], np.int32)
    for exec_mode in (0, 1):
        h = irr.Handle(irr.default_config(map_idx=0, exec=exec_mode))
        h.set_params(irr.moldyn_params(40.0, rc))
        h.set_edges(edges)
        h.set_nodes(pos, 24)
        h.step()
        f = h.get_result(elm_size=12)
        fr = O.lj_reduce_refnum(pos, edges, O.lj_param(rc * rc, 40.0, True))
        assert np.array_equal(f != 0, fr != 0)


def test_wrapped_pairs_with_non_float_side(built_lib, oracle_lib):
    """moldyn's side (N/0.83134)^(1/3) is not a float: pairs across the box
    wall must still match the reference to FP32 accuracy."""
    import irregular_gb300 as irr
    O = oracle_lib
    side = (1048576 / 0.83134) ** 0.3333333  # 108.045548...
    rng = np.random.Generator(np.random.PCG64(3))
    n = 400
    a = (rng.random((n, 3)) * 1.0).astype(np.float32).astype(np.float64)       # near 0
    b = (side - rng.random((n, 3)) * 1.0).astype(np.float32).astype(np.float64)  # near side
    pos = np.concatenate([a, b])
    edges = np.array([[i, n + i] for i in range(n)], np.int32)
    p = O.lj_param(3.5 ** 2, side, True)
    f64, sabs = O.lj_reduce_f64(pos, edges, p)
    fr = O.lj_reduce_refnum(pos, edges, p)
    for exec_mode in (0, 1):
        h = irr.Handle(irr.default_config(map_idx=0, exec=exec_mode))
        h.set_params(irr.moldyn_params(side, 3.5))
        h.set_edges(edges)
        h.set_nodes(pos, 24)
        h.step()
        f = h.get_result(elm_size=12)
        assert scaled_error(f, fr, sabs) <= TOL_VS_REFERENCE
        assert scaled_error(f, f64, sabs) <= TOL_PERNODE_F64


def test_minimd_pbc_map(built_lib, oracle_lib):
    import irregular_gb300 as irr
    O = oracle_lib
    pos32, L = random_box(3000, 0.8442, 21)
    edges = O.neighbor_half_list(pos32, float(L), np.float32(2.8 ** 2))
    pos = pos32.astype(np.float64)
    p = O.lj_param(2.5 ** 2, float(L), True)
    f64, sabs = O.lj_reduce_f64(pos, edges, p)
    for exec_mode in (0, 1):
        h = irr.Handle(irr.default_config(map_idx=irr.IRR_MAP_LJ_MINIMD_PBC, exec=exec_mode))
        h.set_params(irr.minimd_params(2.5 ** 2, float(L)))
        h.set_edges(edges)
        h.set_nodes(pos, 24)
        h.step()
        f = h.get_result(elm_size=12)
        assert normwise_error(f, f64) <= TOL_NORMWISE_F64
        assert scaled_error(f, f64, sabs) <= TOL_PERNODE_F64


def test_set_params_after_init(built_lib, oracle_lib):
    import irregular_gb300 as irr
    O = oracle_lib
    c = load_golden("moldyn_random_2048")
    f, h = run_case(irr, c, exec=1)
    h.set_params(irr.moldyn_params(float(c["side"]), 2.0))
    h.step()
    g = h.get_result(elm_size=12)
    p = O.lj_param(4.0, float(c["side"]), True)
    f64, sabs = O.lj_reduce_f64(c["pos"], c["edges"], p)
    assert normwise_error(g, f64) <= TOL_NORMWISE_F64
    assert not np.array_equal(f, g)


@pytest.mark.parametrize("n", [65536])
def test_larger_random_periodic_properties(built_lib, oracle_lib, n):
    """Config-1 shape (65,536 nodes, ~32 neighbours at 2.5): plain and
    partitioned agree, Newton's third law holds, FP64 error bounds hold."""
    import irregular_gb300 as irr
    O = oracle_lib
    rho = 32.0 / (4.0 / 3.0 * np.pi * 2.5 ** 3)
    pos32, L = random_box(n, rho, 20260001)
    edges = O.neighbor_half_list(pos32, float(L), np.float32(2.5 * 2.5))
    pos = pos32.astype(np.float64)
    p = O.lj_param(6.25, float(L), True)
    f64, sabs = O.lj_reduce_f64(pos, edges, p)
    fr = O.lj_reduce_refnum(pos, edges, p)
    out = {}
    for exec_mode in (0, 1):
        h = irr.Handle(irr.default_config(map_idx=0, exec=exec_mode))
        h.set_params(irr.moldyn_params(float(L), 2.5))
        h.set_edges(edges)
        h.set_nodes(pos, 24)
        h.step()
        out[exec_mode] = h.get_result(elm_size=12)
        assert scaled_error(out[exec_mode], fr, sabs) <= TOL_VS_REFERENCE
        assert normwise_error(out[exec_mode], f64) <= TOL_NORMWISE_F64
        tot = np.abs(out[exec_mode].astype(np.float64).sum(axis=0))
        assert np.all(tot <= 1e-6 * sabs.sum(axis=0))
    assert scaled_error(out[0], out[1], sabs) <= 2 * TOL_PERNODE_F64


@pytest.mark.parametrize("layout", [1, 2])
def test_row_longer_than_a_stage(built_lib, oracle_lib, layout):
    """A hub row of 5999 entries, more than a shared-memory stage holds (5104):
    its work item is read from global memory while the others are staged; CSR
    (1) and sliced (2) layouts both stay on the FP64 oracle."""
    import irregular_gb300 as irr
    O = oracle_lib
    n = 6000
    rho = 32.0 / (4.0 / 3.0 * np.pi * 2.5 ** 3)
    pos32, L = random_box(n, rho, 20260011)
    near = O.neighbor_half_list(pos32, float(L), np.float32(2.5 * 2.5))
    hub = 123
    star = np.stack([np.full(n - 1, hub, np.int32), np.delete(np.arange(n, dtype=np.int32), hub)], axis=1)
    edges = np.concatenate([near, star]).astype(np.int32)
    pos = pos32.astype(np.float64)
    p = O.lj_param(6.25, float(L), True)
    f64, sabs = O.lj_reduce_f64(pos, edges, p)
    h = irr.Handle(irr.default_config(map_idx=0, exec=1, layout=layout))
    h.set_params(irr.moldyn_params(float(L), 2.5))
    h.set_edges(edges)
    h.set_nodes(pos, 24)
    h.step()
    f = h.get_result(elm_size=12)
    assert h.info().layout == layout
    assert normwise_error(f, f64) <= TOL_NORMWISE_F64
    assert scaled_error(f, f64, sabs) <= TOL_PERNODE_F64
    h.close()
