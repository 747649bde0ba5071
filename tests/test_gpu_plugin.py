"""The irregular.h plugin on the GPU: user per-edge functions written in the
reference's irregular.h form (tests/plugin/*/irregular.h), compiled through
the compat shim (compat/irregular/irr_user_map.cu) and run by a partitioned
handle (irr_set_user_map).

Parity:
  * bit for bit against a numpy restatement of the fixture's own arithmetic
    (the plugins are built with -fmad=false, so every FP64 operation rounds
    as numpy's does), for the reduce by the application's `reduce` (first
    insert copied, then reduce in the row's entry order, as the reference's
    reduction objects do: moldyn/irregular/ros.cu:10-68), for a reduce that is
    not + (maximum), and for the compensated (TwoSum) object;
  * the LJ law as a user map against the reference's own results (golden
    fixtures made by the reference's compiled FCPU::map), within the FP32
    reordering tolerance;
  * the compat IrregularRuntime, built without IRR_COMPAT_MAP, running its
    map from the application's tables (moldyn's call sequence).
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import irregular_gb300 as irr
from conftest import PKG, ROOT
from helpers import (TOL_VS_REFERENCE, golden_names, load_golden, oracle_param, random_box,
                     result_errors, scaled_error)
from plugin_build import build_plugins

pytestmark = pytest.mark.gpu

FIXTURES = os.path.join(ROOT, "tests", "plugin")


@pytest.fixture(scope="module")
def plugins(built_lib, tmp_path_factory):
    d = tmp_path_factory.mktemp("plugins")
    jobs = {
        "spring": (os.path.join(FIXTURES, "spring"), str(d / "libspring.so"), True, (), False),
        "spring_comp": (os.path.join(FIXTURES, "spring"), str(d / "libspring_comp.so"), True,
                        ("IRR_PLUGIN_COMPENSATED",), False),
        "lj": (os.path.join(FIXTURES, "lj"), str(d / "liblj.so"), True, (), False),
        "lj_comp": (os.path.join(FIXTURES, "lj"), str(d / "liblj_comp.so"), True,
                    ("IRR_PLUGIN_COMPENSATED", "IRR_PLUGIN_INLINE_MAP=lj_box"), True),
        "lj_obj": (os.path.join(FIXTURES, "lj"), str(d / "lj.o"), False, (), False),
    }
    out = build_plugins(jobs)
    libs = {k: C.CDLL(v) for k, v in out.items() if v.endswith(".so")}
    launch = {k: C.cast(lib.irr_compat_user_launch, C.c_void_p).value for k, lib in libs.items()}
    return {"launch": launch, "libs": libs, "lj_obj": out["lj_obj"]}


# ---------------------------------------------------------------- restatements
def padded_rows(row_off, col):
    n = row_off.shape[0] - 1
    deg = np.diff(row_off).astype(np.int64)
    width = int(deg.max()) if n > 0 and deg.size else 0
    t = np.arange(width)[None, :]
    mask = t < deg[:, None]
    idx = np.where(mask, row_off[:-1, None] + t, 0)
    return np.where(mask, col[idx], 0), mask


def reduce_rows(terms, valid, how):
    """terms (n, w, 3) float32, valid (n, w): the rows' objects in entry order."""
    n, w, _ = terms.shape
    if how == "sum":
        s = np.zeros((n, 3), np.float32)
        c = np.zeros((n, 3), np.float32)
        for t in range(w):
            v = valid[:, t, None]
            a = terms[:, t]
            snew = (s + a).astype(np.float32)
            bb = (snew - s).astype(np.float32)
            e = ((s - (snew - bb).astype(np.float32)).astype(np.float32) + (a - bb).astype(np.float32))
            s = np.where(v, snew, s)
            c = np.where(v, (c + e.astype(np.float32)).astype(np.float32), c)
        return (s + c).astype(np.float32)
    acc = np.zeros((n, 3), np.float32)
    has = np.zeros((n, 1), bool)
    for t in range(w):
        v = valid[:, t, None]
        a = terms[:, t]
        comb = (acc + a).astype(np.float32) if how == "add" else np.fmax(acc, a)
        acc = np.where(v, np.where(has, comb, a), acc)
        has = has | v
    return acc


def spring_terms(x, rows, cols, mask, k, r0, rcut, scale):
    d = x[rows] - x[cols]  # (n, w, 3)
    r2 = d[..., 0] * d[..., 0]
    r2 = r2 + d[..., 1] * d[..., 1]
    r2 = r2 + d[..., 2] * d[..., 2]
    ok = mask & (r2 < rcut * rcut) & (r2 != 0.0)
    with np.errstate(divide="ignore", invalid="ignore"):
        g = (-scale * k) * (1.0 - r0 / np.sqrt(np.where(ok, r2, 1.0)))
    f = (g[..., None] * d).astype(np.float32)
    return f, ok


def lj_terms(x, rows, cols, mask, side=None, cut2=None, cutoff=None):
    d = x[rows] - x[cols]
    if side is not None:
        half = 0.5 * side
        d = np.where(d < -half, d + side, d)
        d = np.where(d > half, d - side, d)
        cut2 = cutoff * cutoff
    rr = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
    ok = mask & (rr < cut2)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        inv = 1.0 / np.where(ok, rr, 1.0)
        inv2 = inv * inv
        inv4 = inv2 * inv2
        s = (inv4 * inv2) * inv - 0.5 * inv4
    return (d * s[..., None]).astype(np.float32), ok


def restate(h, nodes_xyz, terms_fn, how):
    """The plugin kernel's result, in the caller's order, from the handle's
    own partition: node ids are execution-order ids."""
    perm, row_off, col = h.partition()
    x = nodes_xyz[perm]
    n = perm.shape[0]
    cols, mask = padded_rows(row_off, col)
    rows = np.broadcast_to(np.arange(n)[:, None], cols.shape)
    terms, ok = terms_fn(x, rows, cols, mask)
    res = reduce_rows(terms, ok, how)
    out = np.empty_like(res)
    out[perm] = res
    return out


# ---------------------------------------------------------------- cases
def spring_case(n=3000, seed=7):
    rng = np.random.Generator(np.random.PCG64(seed))
    side = (n / 12.0) ** (1.0 / 3.0)
    x = rng.random((n, 3)) * side
    from oracle import oracle as O
    O.build()
    edges = O.neighbor_half_list(x.astype(np.float32), 0.0, np.float32(1.6 ** 2))
    nodes = np.zeros(n, dtype=[("x", np.float64, 3), ("mass", np.float64)])
    nodes["x"] = x
    nodes["mass"] = 1.0 + rng.random(n)
    para = np.array([2.5, 1.0, 1.5], np.float64)  # k, r0, rcut
    return nodes, x, edges, para


def spring_handle(launch, nodes, x, edges, para, coords=True, reorder=1):
    h = irr.Handle(exec=irr.IRR_EXEC_PARTITIONED, reorder=reorder)
    h.set_user_map(launch, 12, 1)
    h.set_params(para)
    h.set_edges(edges)
    h.set_nodes(nodes.view(np.uint8).reshape(len(nodes), -1), elm_size=32)
    if coords:
        h.set_coordinates(x)
    h.init()
    return h


@pytest.mark.parametrize("map_idx,reduce_idx", [(0, 0), (1, 0), (0, 1)])
def test_spring_bit_exact(plugins, map_idx, reduce_idx):
    nodes, x, edges, para = spring_case()
    h = spring_handle(plugins["launch"]["spring"], nodes, x, edges, para)
    h.set_map(map_idx)
    h.set_reduce(reduce_idx)
    h.step()
    got = h.get_result(elm_size=12)
    scale = 2.0 if map_idx == 1 else 1.0
    want = restate(h, x, lambda X, R, Cc, M: spring_terms(X, R, Cc, M, para[0], para[1], para[2], scale),
                   "add" if reduce_idx == 0 else "max")
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # and the FP64 law itself (the float terms' rounding and the float sum)
    if reduce_idx == 0:
        f64 = np.zeros((len(x), 3))
        d = x[edges[:, 0]] - x[edges[:, 1]]
        r = np.sqrt((d * d).sum(1))
        ok = (r < para[2]) & (r > 0)
        g = -scale * para[0] * (1.0 - para[1] / np.where(ok, r, 1.0))
        fe = np.where(ok[:, None], g[:, None] * d, 0.0)
        np.add.at(f64, edges[:, 0], fe)
        np.add.at(f64, edges[:, 1], -fe)
        sabs = np.zeros_like(f64)
        np.add.at(sabs, edges[:, 0], np.abs(fe))
        np.add.at(sabs, edges[:, 1], np.abs(fe))
        assert scaled_error(got, f64, sabs) <= 1e-5


def test_spring_compensated_bit_exact_and_close_to_fp64(plugins):
    nodes, x, edges, para = spring_case(seed=11)
    h = spring_handle(plugins["launch"]["spring_comp"], nodes, x, edges, para)
    h.step()
    got = h.get_result(elm_size=12)
    want = restate(h, x, lambda X, R, Cc, M: spring_terms(X, R, Cc, M, para[0], para[1], para[2], 1.0),
                   "sum")
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # widened read-back (IRR_VALUE_F32 records at twice their size)
    wide = h.get_result(elm_size=24)
    assert np.array_equal(wide, got.astype(np.float64))


def test_spring_caller_order_and_resets(plugins):
    """Records that are not positions and no coordinates: the caller's order
    is kept; reset_node_data and a new edge list both take effect."""
    nodes, x, edges, para = spring_case(n=1500, seed=3)
    h = spring_handle(plugins["launch"]["spring"], nodes, x, edges, para, coords=False)
    perm, _, _ = h.partition(with_entries=False)
    assert np.array_equal(perm, np.arange(len(x)))
    terms = lambda X, R, Cc, M: spring_terms(X, R, Cc, M, para[0], para[1], para[2], 1.0)  # noqa: E731
    h.step()
    assert np.array_equal(h.get_result(elm_size=12), restate(h, x, terms, "add"))
    x2 = x + 0.01
    nodes2 = nodes.copy()
    nodes2["x"] = x2
    h.set_nodes(nodes2.view(np.uint8).reshape(len(nodes2), -1), elm_size=32)
    h.step()
    assert np.array_equal(h.get_result(elm_size=12), restate(h, x2, terms, "add"))
    h.set_edges(edges[: len(edges) // 2])
    h.init()
    h.step()
    assert np.array_equal(h.get_result(elm_size=12), restate(h, x2, terms, "add"))


def test_table_index_out_of_range_fails_loudly(plugins):
    nodes, x, edges, para = spring_case(n=500)
    h = spring_handle(plugins["launch"]["spring"], nodes, x, edges, para)
    h.set_map(2)  # the fixture's table has two maps
    with pytest.raises(irr.IrregularError) as e:
        h.step()
    assert e.value.status == irr.IRR_ERR_ARG
    h.set_map(0)
    h.step()
    h.sync()


@pytest.mark.parametrize("name", golden_names())
def test_lj_user_map_matches_reference(plugins, oracle_lib, name):
    """The LJ law as a user map (tests/plugin/lj): bit for bit against its
    restatement, and within the FP32 reordering tolerance of the reference's
    own result."""
    O = oracle_lib
    c = load_golden(name)
    pos = np.ascontiguousarray(c["pos"], np.float64)
    h = irr.Handle(exec=irr.IRR_EXEC_PARTITIONED)
    h.set_user_map(plugins["launch"]["lj"], 12, 1)
    moldyn = str(c["map"]) == "moldyn"
    if moldyn:
        h.set_params(np.array([float(c["side"]), float(c["cutoff"])], np.float64))
        terms = lambda X, R, Cc, M: lj_terms(X, R, Cc, M, side=float(c["side"]),  # noqa: E731
                                             cutoff=float(c["cutoff"]))
    else:
        h.set_map(1)
        h.set_params(np.array([float(c["param"][0])], np.float64))
        terms = lambda X, R, Cc, M: lj_terms(X, R, Cc, M, cut2=float(c["param"][0]))  # noqa: E731
    h.set_edges(c["edges"])
    h.set_nodes(pos, elm_size=24)
    h.init()
    h.step()
    got = h.get_result(elm_size=12)
    assert np.array_equal(got.view(np.uint32), restate(h, pos, terms, "add").view(np.uint32))
    _, sabs = O.lj_reduce_f64(pos, c["edges"], oracle_param(O, c))
    assert scaled_error(got, c["f_ref"], sabs) <= TOL_VS_REFERENCE


def test_compat_runtime_runs_the_application_map(plugins, oracle_lib, tmp_path):
    """moldyn's call sequence through the compat IrregularRuntime with no
    IRR_COMPAT_MAP: the map comes from the application's table."""
    O = oracle_lib
    exe = str(tmp_path / "moldyn_like_plugin")
    cuda_lib = "/usr/local/cuda/lib64"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(PKG, "compat"), "-I",
                        os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "drop_in", "moldyn_like.cpp"),
                        plugins["lj_obj"], "-o", exe, "-L", PKG, "-lirregular_gb300", f"-Wl,-rpath,{PKG}",
                        "-L", cuda_lib, "-lcudart", f"-Wl,-rpath,{cuda_lib}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    c = load_golden("moldyn_random_2048")
    inp, out = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    n, e = c["pos"].shape[0], c["edges"].shape[0]
    with open(inp, "wb") as f:
        np.array([n, e], np.int64).tofile(f)
        np.asarray(c["param"], np.float64).tofile(f)
        np.ascontiguousarray(c["pos"], np.float64).tofile(f)
        np.ascontiguousarray(c["edges"], np.int32).tofile(f)
    r = subprocess.run([exe, inp, out, "3"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    forces = np.fromfile(out, np.float32).reshape(n, 3)
    _, sabs = O.lj_reduce_f64(c["pos"], c["edges"], oracle_param(O, c))
    assert scaled_error(forces, c["f_ref"], sabs) <= TOL_VS_REFERENCE


def test_user_map_handles_run_alone(plugins):
    """A batch runs the library's tiled kernel: a handle with a user map is
    refused when the batch is finalised."""
    nodes, x, edges, para = spring_case(n=400)
    h = spring_handle(plugins["launch"]["spring"], nodes, x, edges, para)
    b = irr.Batch()
    b.add(h)
    with pytest.raises(irr.IrregularError) as e:
        b.finalize()
    assert e.value.status == irr.IRR_ERR_STATE


def test_user_map_on_shards(plugins):
    """A user map on shard handles (irr_set_shard): the union of the shards'
    owned rows equals one whole-problem handle bit for bit."""
    import sharding
    nodes, x, edges, para = spring_case(n=2500, seed=21)
    hw = spring_handle(plugins["launch"]["spring"], nodes, x, edges, para)
    hw.step()
    perm, row_off, col = hw.partition()
    whole = hw.get_result(elm_size=12)[perm]
    rec = nodes.view(np.uint8).reshape(len(nodes), -1)[perm]
    got = np.zeros_like(whole)
    for sh in sharding.plan(row_off, col, 3):
        lp = sharding.local_problem(sh, row_off, col)
        h = irr.Handle(exec=irr.IRR_EXEC_PARTITIONED, reorder=0)
        h.set_user_map(plugins["launch"]["spring"], 12, 1)
        h.set_params(para)
        h.set_shard(lp.own_lo, lp.own_hi)
        h.set_edges(lp.edges)
        h.set_nodes(np.ascontiguousarray(rec[lp.nodes]), elm_size=32)
        h.init()
        h.step()
        got[lp.lo:lp.hi] = h.get_result(elm_size=12)
    assert np.array_equal(got.view(np.uint32), whole.view(np.uint32))


def test_user_map_without_edges(plugins):
    """No edges: every row's object stays empty and stores zero bytes."""
    nodes, x, _, para = spring_case(n=64, seed=2)
    h = spring_handle(plugins["launch"]["spring"], nodes, x, np.zeros((0, 2), np.int32), para)
    h.step()
    assert np.all(h.get_result(elm_size=12) == 0)


@pytest.mark.parametrize("user", [False, True])
def test_python_irregular_runtime(plugins, oracle_lib, user):
    """The ctypes IrregularRuntime mirror with moldyn's call sequence, on a
    built-in law and on the application's map (the LJ fixture)."""
    O = oracle_lib
    c = load_golden("moldyn_random_2048")
    pos = np.ascontiguousarray(c["pos"], np.float64)
    n, e = pos.shape[0], c["edges"].shape[0]
    kw = dict(user_launch=plugins["launch"]["lj"], value_size=12) if user else {}
    rt = irr.IrregularRuntime(e, n, c["edges"], None, pos, 0, 24, 12, 3, pos, 8,
                              parameter=np.asarray(c["param"], np.float64), parameter_size=16, **kw)
    rt.IrregularInit()
    for _ in range(2):
        rt.reset_node_data(pos)
        rt.IrregularStart()
        f = rt.get_reduction_result()
        rt.IrregularBarrier()
    _, sabs = O.lj_reduce_f64(pos, c["edges"], oracle_param(O, c))
    assert scaled_error(f, c["f_ref"], sabs) <= TOL_VS_REFERENCE


def test_fp64_user_map_error_quantiles(plugins, oracle_lib):
    """The precise path: the LJ law in FP64 as a user map, its float terms
    summed with compensated (TwoSum) accumulators.  Against FP64 per result
    (|df|inf / max(|f64|inf, 2^-10 sum_e |f_e|inf)) over all 65,536 nodes of
    a ~64-neighbour box: the median and the 99th percentile are far below
    1e-6, and the worst node is bounded by the float VALUE terms themselves
    (each rounded to 2^-24 of its size) where a node's forces cancel to
    near the 2^-10 floor -- no law can do better with float terms."""
    O = oracle_lib
    pos32, L = random_box(65536, 64.0 / (4.0 / 3.0 * np.pi * 2.5 ** 3), 909)
    edges = O.neighbor_half_list(pos32, float(L), np.float32(2.5 * 2.5))
    pos = pos32.astype(np.float64)
    h = irr.Handle(exec=irr.IRR_EXEC_PARTITIONED)
    h.set_user_map(plugins["launch"]["lj_comp"], 12, 1)
    h.set_params(np.array([float(L), 2.5], np.float64))
    h.set_edges(edges)
    h.set_nodes(pos, elm_size=24)
    h.init()
    h.step()
    f = h.get_result(elm_size=12)
    p = O.lj_param(2.5 * 2.5, float(L), True)
    f64, _ = O.lj_reduce_f64(pos, edges, p)
    sinf = O.lj_edge_scale_inf(pos, edges, p)
    r = result_errors(f, f64, sinf)
    q = (np.percentile(r, 50), np.percentile(r, 99), r.max())
    assert q[0] <= 1e-7 and q[1] <= 1e-6 and q[2] <= 1e-5, q
    # the worst node is bounded by its float terms: redo it with the FP64
    # terms rounded to float and summed exactly
    worst = int(np.argmax(r))
    inc = edges[(edges[:, 0] == worst) | (edges[:, 1] == worst)]
    d = pos[inc[:, 0]] - pos[inc[:, 1]]
    d = np.where(d < -0.5 * L, d + L, d)
    d = np.where(d > 0.5 * L, d - L, d)
    rd = (d * d).sum(axis=1)
    ok = rd < 2.5 * 2.5
    s_ = np.where(ok, 1.0 / np.where(ok, rd, 1.0) ** 7 - 0.5 / np.where(ok, rd, 1.0) ** 4, 0.0)
    fe = (d * s_[:, None]).astype(np.float32).astype(np.float64)
    sign = np.where(inc[:, 0] == worst, 1.0, -1.0)[:, None]
    rounded_only = result_errors((fe * sign).sum(axis=0)[None], f64[worst][None], sinf[worst:worst + 1])[0]
    assert r[worst] <= 2 * rounded_only + 1e-12, (r[worst], rounded_only)
