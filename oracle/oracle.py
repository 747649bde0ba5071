"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import
this module, and only for reference results to compare against or the timed
CPU baseline; the product library never does.  It loads

  oracle/liboracle.so          the C restatement of the reference's CPU path
                               (irr_oracle.c; provenance in irr_oracle.h), and
  oracle/_ref/libref_*.so      the reference's own CPU code compiled from its
                               sources (ref_harness.cpp), when it was built.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_lib = None
_ref = {}


class LJParam(C.Structure):
    _fields_ = [("side", C.c_double), ("cutoff2", C.c_double), ("periodic", C.c_int)]


def reference_tree() -> str:
    """Where the reference's sources are read from: $IRR_REFERENCE_TREE, else the
    `REF ?=` default of oracle/Makefile (the recipe that compiles them).  The
    tree may be absent; callers check before using it."""
    env = os.environ.get("IRR_REFERENCE_TREE")
    if env:
        return env
    try:
        with open(os.path.join(HERE, "Makefile")) as f:
            for line in f:
                key, sep, val = line.partition("?=")
                if sep and key.strip() == "REF":
                    return val.strip()
    except OSError:
        pass
    return ""


def build(quiet: bool = True) -> None:
    """Compiles liboracle.so with the committed Makefile."""
    out = subprocess.run(["make", "-C", HERE, "liboracle.so"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        i64 = C.c_int64
        L.orc_lj_reduce_f64.argtypes = [i64, P, i64, P, C.POINTER(LJParam), P, P]
        L.orc_lj_reduce_refnum_f32.argtypes = [i64, P, i64, P, C.POINTER(LJParam), P]
        L.orc_lj_edge_scale_inf.argtypes = [i64, P, i64, P, C.POINTER(LJParam), P]
        L.orc_cpu_executor.argtypes = [i64, P, i64, P, C.POINTER(LJParam), C.c_int, i64, P,
                                       C.POINTER(C.c_double)]
        L.orc_cpu_executor.restype = C.c_int
        L.orc_exec_create.argtypes = [i64, C.c_int]
        L.orc_exec_create.restype = P
        L.orc_exec_run.argtypes = [P, P, i64, P, C.POINTER(LJParam), i64, P]
        L.orc_exec_run.restype = C.c_double
        L.orc_exec_destroy.argtypes = [P]
        L.orc_neighbor_half_list.argtypes = [i64, P, C.c_float, C.c_float, P, i64]
        L.orc_neighbor_half_list.restype = i64
        L.orc_neighbor_half_list_rows.argtypes = [i64, P, C.c_float, C.c_float, i64, i64, P, i64]
        L.orc_neighbor_half_list_rows.restype = i64
        L.orc_md_run.argtypes = [i64, P, P, C.c_double, C.c_double, C.c_double, C.c_double,
                                 C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_md_run.restype = C.c_int
        L.orc_md_run_mt.argtypes = [i64, P, P, C.c_double, C.c_double, C.c_double, C.c_double,
                                    C.c_int, C.c_int, C.POINTER(C.c_double),
                                    C.POINTER(C.c_double), C.c_int, C.c_int]
        L.orc_md_run_mt.restype = C.c_int
        L.orc_fcc_moldyn.argtypes = [C.c_int, C.c_double, P]
        L.orc_fcc_minimd.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, P, i64]
        L.orc_fcc_minimd.restype = i64
        L.orc_morton_keys.argtypes = [i64, P, P, P, P]
        L.orc_partition.argtypes = [i64, P, P, P, i64, P, P, P, P, P]
        L.orc_partition.restype = C.c_int
        L.orc_hilbert_keys.argtypes = [i64, P, P, P, P]
        L.orc_partition_curve.argtypes = [i64, P, P, P, C.c_int, i64, P, P, P, P, P]
        L.orc_partition_curve.restype = C.c_int
        L.orc_staged_layout.argtypes = [i64, P, P, C.c_int, C.c_int, C.c_int,
                                        C.POINTER(i64), C.POINTER(i64), C.POINTER(i64),
                                        P, P, P, P]
        L.orc_staged_layout.restype = C.c_int
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def lj_param(cutoff2: float, side: float = 0.0, periodic: bool = False) -> LJParam:
    return LJParam(float(side), float(cutoff2), 1 if periodic else 0)


def _pos64(pos) -> np.ndarray:
    return np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)


def _edges(edges) -> np.ndarray:
    return np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)


def lj_reduce_f64(pos, edges, param: LJParam):
    """FP64 oracle forces and the per-node absolute-term scale."""
    pos = _pos64(pos)
    edges = _edges(edges)
    n = pos.shape[0]
    f = np.zeros((n, 3), np.float64)
    s = np.zeros((n, 3), np.float64)
    lib().orc_lj_reduce_f64(n, _p(pos), edges.shape[0], _p(edges), C.byref(param), _p(f), _p(s))
    return f, s


def lj_edge_scale_inf(pos, edges, param: LJParam) -> np.ndarray:
    """Per node: the sum over its in-cutoff edges of max_c |f_e,c| (FP64), the
    scale of the per-result error metric (helpers.result_error)."""
    pos = _pos64(pos)
    edges = _edges(edges)
    n = pos.shape[0]
    s = np.zeros(n, np.float64)
    lib().orc_lj_edge_scale_inf(n, _p(pos), edges.shape[0], _p(edges), C.byref(param), _p(s))
    return s


def lj_reduce_refnum(pos, edges, param: LJParam) -> np.ndarray:
    """The reference's CPU numerics (FP64 per edge, float accumulate, edge order)."""
    pos = _pos64(pos)
    edges = _edges(edges)
    n = pos.shape[0]
    f = np.zeros((n, 3), np.float32)
    lib().orc_lj_reduce_refnum_f32(n, _p(pos), edges.shape[0], _p(edges), C.byref(param), _p(f))
    return f


def cpu_executor(pos, edges, param: LJParam, threads: int, chunk: int = 1000000):
    """Port of the reference's pthread executor; returns (forces, seconds)."""
    pos = _pos64(pos)
    edges = _edges(edges)
    n = pos.shape[0]
    f = np.zeros((n, 3), np.float32)
    secs = C.c_double(0.0)
    rc = lib().orc_cpu_executor(n, _p(pos), edges.shape[0], _p(edges), C.byref(param),
                                int(threads), int(chunk), _p(f), C.byref(secs))
    if rc != 0:
        raise RuntimeError("orc_cpu_executor failed")
    return f, secs.value


class Executor:
    """Reusable executor port (tables allocated once) for timed passes."""

    def __init__(self, n: int, threads: int):
        self.n = int(n)
        self.threads = int(threads)
        self._h = lib().orc_exec_create(self.n, self.threads)
        if not self._h:
            raise MemoryError("orc_exec_create failed")

    def run(self, pos32: np.ndarray, edges: np.ndarray, param: LJParam, chunk: int = 1000000,
            out: np.ndarray | None = None) -> float:
        pos32 = np.ascontiguousarray(pos32, np.float32)
        edges = _edges(edges)
        ptr = _p(out) if out is not None else None
        s = lib().orc_exec_run(self._h, _p(pos32), edges.shape[0], _p(edges), C.byref(param),
                               int(chunk), ptr)
        if s < 0:
            raise RuntimeError("orc_exec_run failed")
        return s

    def close(self):
        if self._h:
            lib().orc_exec_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def neighbor_half_list(pos32, box: float, list_cut2: float) -> np.ndarray:
    """Half list (i<j, sorted) with the float criterion shared with the GPU builder."""
    pos32 = np.ascontiguousarray(pos32, np.float32).reshape(-1, 3)
    n = pos32.shape[0]
    L = lib()
    cnt = L.orc_neighbor_half_list(n, _p(pos32), float(box), float(list_cut2), None, 0)
    if cnt < 0:
        raise ValueError("bad neighbour-list arguments")
    out = np.zeros((max(cnt, 0), 2), np.int32)
    if cnt:
        L.orc_neighbor_half_list(n, _p(pos32), float(box), float(list_cut2), _p(out), cnt)
    return out


def neighbor_half_list_rows(pos32, box: float, list_cut2: float, row_begin: int,
                            row_end: int) -> np.ndarray:
    """Rows [row_begin, row_end) of the half list: a bounded sample of a large list."""
    pos32 = np.ascontiguousarray(pos32, np.float32).reshape(-1, 3)
    n = pos32.shape[0]
    L = lib()
    cnt = L.orc_neighbor_half_list_rows(n, _p(pos32), float(box), float(list_cut2), row_begin,
                                        row_end, None, 0)
    if cnt < 0:
        raise ValueError("bad neighbour-list arguments")
    out = np.zeros((max(cnt, 0), 2), np.int32)
    if cnt:
        L.orc_neighbor_half_list_rows(n, _p(pos32), float(box), float(list_cut2), row_begin,
                                      row_end, _p(out), cnt)
    return out


def neighbor_count(pos32, box: float, list_cut2: float) -> int:
    pos32 = np.ascontiguousarray(pos32, np.float32).reshape(-1, 3)
    return int(lib().orc_neighbor_half_list(pos32.shape[0], _p(pos32), float(box),
                                            float(list_cut2), None, 0))


def md_run(pos, vel, side: float, cutforce: float, skin: float, dt: float, steps: int,
           rebuild_every: int, threads: int = 0, float_forces: bool = False):
    """FP64 reference MD; returns (pos, vel, kinetic, potential).  threads = 0:
    all host cores (the list is the serial one; forces are summed per thread
    in a fixed order, FP64 to ~1e-16).  float_forces: evaluate the (FP64) forces
    at the float copy of the positions, as the GPU's FP32 reduction does, so
    that a comparison isolates the per-edge FP32 arithmetic."""
    p = np.array(pos, np.float64).reshape(-1, 3).copy()
    v = np.array(vel, np.float64).reshape(-1, 3).copy()
    ke, pe = C.c_double(), C.c_double()
    if threads <= 0:
        threads = min(os.cpu_count() or 1, 32)
    rc = lib().orc_md_run_mt(p.shape[0], _p(p), _p(v), float(side), float(cutforce), float(skin),
                             float(dt), int(steps), int(rebuild_every), C.byref(ke), C.byref(pe),
                             int(threads), int(bool(float_forces)))
    if rc != 0:
        raise ValueError("orc_md_run failed")
    return p, v, ke.value, pe.value


def fcc_moldyn(m: int, side: float) -> np.ndarray:
    pos = np.zeros((4 * m ** 3, 3), np.float64)
    lib().orc_fcc_moldyn(int(m), float(side), _p(pos))
    return pos


def fcc_minimd(nx: int, ny: int, nz: int, rho: float) -> np.ndarray:
    L = lib()
    cnt = L.orc_fcc_minimd(nx, ny, nz, float(rho), None, 0)
    pos = np.zeros((cnt, 3), np.float64)
    L.orc_fcc_minimd(nx, ny, nz, float(rho), _p(pos), cnt)
    return pos


def morton_keys(pos32, lo, scale) -> np.ndarray:
    pos32 = np.ascontiguousarray(pos32, np.float32).reshape(-1, 3)
    lo = np.ascontiguousarray(lo, np.float32)
    scale = np.ascontiguousarray(scale, np.float32)
    keys = np.zeros(pos32.shape[0], np.uint32)
    lib().orc_morton_keys(pos32.shape[0], _p(pos32), _p(lo), _p(scale), _p(keys))
    return keys


def hilbert_keys(pos32, lo, scale) -> np.ndarray:
    pos32 = np.ascontiguousarray(pos32, np.float32).reshape(-1, 3)
    lo = np.ascontiguousarray(lo, np.float32)
    scale = np.ascontiguousarray(scale, np.float32)
    keys = np.zeros(pos32.shape[0], np.uint32)
    lib().orc_hilbert_keys(pos32.shape[0], _p(pos32), _p(lo), _p(scale), _p(keys))
    return keys


def partition(pos32, lo, scale, edges, curve: str = "morton"):
    """Returns (perm, inv, row_off, col) of the bit-exact partition oracle;
    nodes ordered along the Morton or the Hilbert curve."""
    pos32 = np.ascontiguousarray(pos32, np.float32).reshape(-1, 3)
    edges = _edges(edges)
    n = pos32.shape[0]
    e = edges.shape[0]
    lo = np.ascontiguousarray(lo, np.float32)
    scale = np.ascontiguousarray(scale, np.float32)
    perm = np.zeros(n, np.int32)
    inv = np.zeros(n, np.int32)
    row_off = np.zeros(n + 1, np.int64)
    col = np.zeros(max(2 * e, 1), np.int32)
    rc = lib().orc_partition_curve(n, _p(pos32), _p(lo), _p(scale), 0 if curve == "hilbert" else 1,
                                   e, _p(edges), _p(perm), _p(inv), _p(row_off), _p(col))
    if rc != 0:
        raise ValueError(f"orc_partition failed ({rc})")
    return perm, inv, row_off, col[: 2 * e]


def staged_layout(row_off, col, slices_per_item: int = 8, tab_max: int = 640,
                  stream_max: int = 3584):
    """The staged ("halo") layout of a CSR (orc_staged_layout): a dict of items
    (k, 6: row0, nrows, word0, nwords, tab0, ntab), slice_off, words and ids, or
    None when a slice alone does not fit the limits."""
    row_off = np.ascontiguousarray(row_off, np.int64)
    col = np.ascontiguousarray(col, np.int32)
    n = row_off.shape[0] - 1
    ni, nw, nd = C.c_int64(), C.c_int64(), C.c_int64()
    L = lib()
    rc = L.orc_staged_layout(n, _p(row_off), _p(col), slices_per_item, tab_max, stream_max,
                             C.byref(ni), C.byref(nw), C.byref(nd), None, None, None, None)
    if rc == -1:
        return None
    if rc != 0:
        raise ValueError(f"orc_staged_layout failed ({rc})")
    items = np.zeros((max(ni.value, 1), 6), np.int32)
    slice_off = np.zeros((n + 7) // 8 + 1, np.uint32)
    words = np.zeros(max(nw.value, 1), np.uint32)
    ids = np.zeros(max(nd.value, 1), np.int32)
    rc = L.orc_staged_layout(n, _p(row_off), _p(col), slices_per_item, tab_max, stream_max,
                             C.byref(ni), C.byref(nw), C.byref(nd), _p(items), _p(slice_off),
                             _p(words), _p(ids))
    if rc != 0:
        raise ValueError(f"orc_staged_layout failed ({rc})")
    return {"items": items[: ni.value], "slice_off": slice_off, "words": words[: nw.value],
            "ids": ids[: nd.value]}


def morton_frame(pos32):
    """The quantisation frame the product partitioner uses: lo = per-axis min,
    scale = 1024 / (max - min) in float (0 for a flat axis)."""
    pos32 = np.ascontiguousarray(pos32, np.float32).reshape(-1, 3)
    if pos32.shape[0] == 0:
        return np.zeros(3, np.float32), np.zeros(3, np.float32)
    lo = pos32.min(axis=0).astype(np.float32)
    hi = pos32.max(axis=0).astype(np.float32)
    ext = (hi - lo).astype(np.float32)
    scale = np.where(ext > 0, np.float32(1024.0) / np.where(ext > 0, ext, np.float32(1)),
                     np.float32(0)).astype(np.float32)
    return lo, scale


# ---------------------------------------------------------------- reference

def ref_available(which: str = "moldyn") -> bool:
    return os.path.exists(os.path.join(REF_DIR, f"libref_{which}.so"))


def ref_lib(which: str = "moldyn"):
    if which not in _ref:
        path = os.path.join(REF_DIR, f"libref_{which}.so")
        L = C.CDLL(path)
        P = C.c_void_p
        L.ref_map_all.argtypes = [C.c_int64, P, C.c_int64, P, P, P]
        L.ref_map_all.restype = C.c_int
        L.ref_compute_cpu.argtypes = [C.c_int64, P, C.c_int64, P, P, C.c_int, C.c_int, P,
                                      C.POINTER(C.c_double)]
        L.ref_compute_cpu.restype = C.c_int
        L.ref_num_buckets.restype = C.c_int
        _ref[which] = L
    return _ref[which]


def ref_param_bytes(which: str, cutoff: float, side: float = 0.0) -> np.ndarray:
    """The reference's parameter blob: moldyn `struct para {double side;
    double cutoffRadius;}` (moldyn/moldyn.h:39-43); miniMD `double
    cutforcesq` (miniMD/ljs.cu:123)."""
    if which == "moldyn":
        return np.array([side, cutoff], np.float64)
    return np.array([cutoff * cutoff], np.float64)


def ref_map_all(which: str, pos, edges, param_blob: np.ndarray) -> np.ndarray:
    pos = _pos64(pos)
    edges = _edges(edges)
    n = pos.shape[0]
    out = np.zeros((n, 3), np.float32)
    rc = ref_lib(which).ref_map_all(n, _p(pos), edges.shape[0], _p(edges), _p(param_blob),
                                    _p(out))
    if rc != 0:
        raise RuntimeError("ref_map_all failed")
    return out


def ref_compute_cpu(which: str, pos, edges, param_blob: np.ndarray, threads: int):
    pos = _pos64(pos)
    edges = _edges(edges)
    n = pos.shape[0]
    out = np.zeros((n, 3), np.float32)
    secs = C.c_double(0)
    rc = ref_lib(which).ref_compute_cpu(n, _p(pos), edges.shape[0], _p(edges), _p(param_blob),
                                        int(param_blob.nbytes), int(threads), _p(out),
                                        C.byref(secs))
    if rc != 0:
        raise RuntimeError("ref_compute_cpu failed")
    return out, secs.value


def ref_read_graph(path: str, max_edges: int) -> np.ndarray:
    """moldyn's own ReadInputGraph (moldyn/misc.c:62-146, built by `make ref`):
    the half list it returns, as int32 pairs.  The reference exits the process
    on an unreadable file or an edge-count mismatch, so call it only on files
    it accepts; `max_edges` bounds its output buffer."""
    L = C.CDLL(os.path.join(REF_DIR, "libref_misc.so"))
    L.ReadInputGraph.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_void_p]
    L.ReadInputGraph.restype = None
    n, m = C.c_int(0), C.c_int(0)
    el = np.full((max(max_edges, 1), 2), -1, np.int32)
    L.ReadInputGraph(path.encode(), C.byref(n), C.byref(m), _p(el))
    return el[: m.value].copy(), n.value


def ref_read_coords(path: str, n: int) -> np.ndarray:
    """moldyn's own ReadCoord (moldyn/misc.c:224-246): n xyz triples in double."""
    L = C.CDLL(os.path.join(REF_DIR, "libref_misc.so"))
    L.ReadCoord.argtypes = [C.c_char_p, C.c_int, C.c_void_p]
    L.ReadCoord.restype = None
    xyz = np.zeros((max(n, 1), 3), np.float64)
    L.ReadCoord(path.encode(), int(n), _p(xyz))
    return xyz[:n].copy()
