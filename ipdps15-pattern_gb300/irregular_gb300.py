"""Python host binding of libirregular_gb300.so (ctypes over the C ABI).

`IrregularRuntime` mirrors the reference's C++ class of the same name
(moldyn/irregular/irregular_runtime.h:12-112): construct it with the edge
list, node data and parameter block, call IrregularInit(), then per iteration
reset_node_data() / IrregularStart() / get_reduction_result().  Errors raise
IrregularError carrying the C status code; nothing falls back to the CPU.  If
the shared library has not been built the import of this module still works,
but the first call raises with the build instruction.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# IRR_LIBRARY selects another build of the library (e.g. a variant build).
LIB_PATH = os.environ.get("IRR_LIBRARY") or os.path.join(HERE, "libirregular_gb300.so")

IRR_OK = 0
IRR_ERR_ARG = 1
IRR_ERR_INDEX = 2
IRR_ERR_STATE = 3
IRR_ERR_CUDA = 4
IRR_ERR_NOMEM = 5
IRR_ERR_CAPACITY = 6
IRR_ERR_DEVICE = 7
IRR_ERR_BUDGET = 8

IRR_MAP_LJ_MOLDYN = 0
IRR_MAP_LJ_MINIMD = 1
IRR_MAP_LJ_MINIMD_PBC = 2
IRR_REDUCE_SUM = 0
IRR_EXEC_PLAIN = 0
IRR_EXEC_PARTITIONED = 1
IRR_ORDER_HILBERT = 0
IRR_ORDER_MORTON = 1
IRR_LAYOUT_AUTO = 0
IRR_LAYOUT_CSR = 1
IRR_LAYOUT_SLICED = 2
IRR_LAYOUT_STAGED = 3


class IrregularError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[status {status}] {msg}")
        self.status = status


class Config(C.Structure):
    _fields_ = [("device", C.c_int), ("exec", C.c_int), ("map_idx", C.c_int),
                ("reduce_idx", C.c_int), ("block_nodes", C.c_int), ("lanes_per_row", C.c_int),
                ("reorder", C.c_int), ("stage_smem", C.c_int), ("layout", C.c_int),
                ("order", C.c_int), ("wait_limit_us", C.c_int), ("reserved", C.c_int * 5)]


class Info(C.Structure):
    _fields_ = [("num_nodes", C.c_int64), ("num_edges", C.c_int64), ("num_entries", C.c_int64),
                ("num_blocks", C.c_int64), ("device_bytes", C.c_int64),
                ("block_nodes", C.c_int32), ("lanes_per_row", C.c_int32),
                ("stage_smem", C.c_int32), ("exec", C.c_int32), ("layout", C.c_int32),
                ("order", C.c_int32), ("num_slots", C.c_int64), ("own_lo", C.c_int64),
                ("own_hi", C.c_int64)]


class MDConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("rebuild_every", C.c_int), ("dt", C.c_double),
                ("cutforce", C.c_double), ("skin", C.c_double), ("side", C.c_double),
                ("reorder_every", C.c_int), ("exec_plain", C.c_int), ("row_slots", C.c_int),
                ("reserved", C.c_int * 5)]


class MDInfo(C.Structure):
    _fields_ = [("num_atoms", C.c_int64), ("num_edges", C.c_int64), ("steps", C.c_int64),
                ("rebuilds", C.c_int64)]


class BatchInfo(C.Structure):
    _fields_ = [("num_instances", C.c_int64), ("num_nodes", C.c_int64), ("num_edges", C.c_int64),
                ("num_items", C.c_int64), ("lanes_per_row", C.c_int32),
                ("block_nodes", C.c_int32), ("graph", C.c_int32), ("reserved", C.c_int32)]


class ServeConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("num_jobs", C.c_int), ("steps_per_job", C.c_int),
                ("rebuild_every", C.c_int), ("mode", C.c_int), ("only_job", C.c_int),
                ("max_resident", C.c_int), ("reserved0", C.c_int), ("arrival_rate", C.c_double),
                ("density", C.c_double), ("cutforce", C.c_double), ("skin", C.c_double),
                ("dt", C.c_double), ("temperature", C.c_double), ("min_atoms", C.c_int64),
                ("max_atoms", C.c_int64), ("budget_bytes", C.c_double), ("seed", C.c_uint64),
                ("policy", C.c_int), ("reserved", C.c_int * 7)]


class ServeStats(C.Structure):
    _fields_ = [("jobs_done", C.c_int64), ("rejected", C.c_int64), ("max_resident", C.c_int64),
                ("reserved0", C.c_int64), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("mean_ms", C.c_double), ("max_ms", C.c_double), ("makespan_s", C.c_double),
                ("pair_evals", C.c_double), ("edges_per_s", C.c_double),
                ("peak_budget_bytes", C.c_double)]


class ServeJob(C.Structure):
    _fields_ = [("atoms", C.c_int64), ("edges", C.c_int64), ("arrival_s", C.c_double),
                ("admit_s", C.c_double), ("done_s", C.c_double), ("energy", C.c_double),
                ("state_hash", C.c_uint64), ("status", C.c_int32), ("reserved", C.c_int32)]


IRR_SERVE_CONTINUOUS = 0
IRR_SERVE_SERIAL = 1
IRR_SERVE_SERIAL_PLAIN = 2
IRR_SERVE_FIFO = 0
IRR_SERVE_SJF = 1


# name -> (restype, argtypes); every symbol include/irregular_gb300.h declares
P = C.c_void_p
I64 = C.c_int64
_SIGS = {
    "irr_config_default": (None, [C.POINTER(Config)]),
    "irr_status_string": (C.c_char_p, [C.c_int]),
    "irr_create": (C.c_int, [C.POINTER(Config), C.POINTER(P)]),
    "irr_destroy": (C.c_int, [P]),
    "irr_last_error": (C.c_char_p, [P]),
    "irr_set_stream": (C.c_int, [P, P]),
    "irr_set_map": (C.c_int, [P, C.c_int]),
    "irr_set_reduce": (C.c_int, [P, C.c_int]),
    "irr_set_params": (C.c_int, [P, P, C.c_int]),
    "irr_set_edges": (C.c_int, [P, P, I64]),
    "irr_set_edges_device": (C.c_int, [P, P, I64]),
    "irr_set_nodes": (C.c_int, [P, P, C.c_int, I64]),
    "irr_set_nodes_device": (C.c_int, [P, P, C.c_int, I64]),
    "irr_init": (C.c_int, [P]),
    "irr_step": (C.c_int, [P]),
    "irr_get_result": (C.c_int, [P, P, C.c_int]),
    "irr_get_result_device": (C.c_int, [P, P, C.c_int]),
    "irr_sync": (C.c_int, [P]),
    "irr_set_wait_limit": (C.c_int, [P, I64, C.c_int]),
    "irr_get_info": (C.c_int, [P, C.POINTER(Info)]),
    "irr_get_partition": (C.c_int, [P, P, P, P]),
    "irr_get_staged": (C.c_int, [P, P, P, P, P, P]),
    "irr_set_user_map": (C.c_int, [P, P, P, C.c_int, C.c_int]),
    "irr_set_coordinates": (C.c_int, [P, P, C.c_int, C.c_int, I64]),
    "irr_set_shard": (C.c_int, [P, I64, I64]),
    "irr_step_pipelined": (C.c_int, [P, P, C.c_int, P, C.c_int]),
    "irr_pipeline_sync": (C.c_int, [P]),
    "irr_set_nodes_range": (C.c_int, [P, P, C.c_int, I64, I64]),
    "irr_set_nodes_range_device": (C.c_int, [P, P, C.c_int, I64, I64]),
    "irr_neighbor_build": (C.c_int, [C.c_int, P, P, C.c_int, C.c_int, I64, C.c_float, C.c_float,
                                     C.POINTER(P), C.POINTER(I64)]),
    "irr_device_free": (C.c_int, [C.c_int, P]),
    "irr_morton_order_static": (C.c_int, [C.c_int, P, P, C.c_int, I64, P]),
    "irr_read_graph": (C.c_int, [C.c_char_p, C.POINTER(I64), C.POINTER(I64), P, I64, C.c_int]),
    "irr_read_coords": (C.c_int, [C.c_char_p, I64, P]),
    "irr_write_graph": (C.c_int, [C.c_char_p, I64, P, I64]),
    "irr_write_coords": (C.c_int, [C.c_char_p, I64, P]),
    "irr_batch_create": (C.c_int, [C.c_int, C.POINTER(P)]),
    "irr_batch_destroy": (C.c_int, [P]),
    "irr_batch_last_error": (C.c_char_p, [P]),
    "irr_batch_set_stream": (C.c_int, [P, P]),
    "irr_batch_add": (C.c_int, [P, P]),
    "irr_batch_finalize": (C.c_int, [P, C.c_int]),
    "irr_batch_step": (C.c_int, [P]),
    "irr_batch_capture": (C.c_int, [P]),
    "irr_batch_sync": (C.c_int, [P]),
    "irr_batch_get_info": (C.c_int, [P, C.POINTER(BatchInfo)]),
    "irr_autotune": (C.c_int, [P]),
    "irr_serve_config_default": (None, [C.POINTER(ServeConfig)]),
    "irr_serve_run": (C.c_int, [C.POINTER(ServeConfig), C.POINTER(ServeStats), P]),
    "irr_serve_job_state": (C.c_int, [C.POINTER(ServeConfig), C.c_int, C.POINTER(I64),
                                      C.POINTER(C.c_double), P, P]),
    "irr_md_config_default": (None, [C.POINTER(MDConfig)]),
    "irr_md_create": (C.c_int, [C.POINTER(MDConfig), P, P, I64, C.POINTER(P)]),
    "irr_md_destroy": (C.c_int, [P]),
    "irr_md_last_error": (C.c_char_p, [P]),
    "irr_md_set_stream": (C.c_int, [P, P]),
    "irr_md_run": (C.c_int, [P, C.c_int]),
    "irr_md_energy": (C.c_int, [P, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                C.POINTER(C.c_double)]),
    "irr_md_get_state": (C.c_int, [P, P, P]),
    "irr_md_get_forces": (C.c_int, [P, P]),
    "irr_md_get_info": (C.c_int, [P, C.POINTER(MDInfo)]),
}

_lib = None


def lib_path() -> str:
    return LIB_PATH


def load():
    """Loads the CUDA library; raises if it was never built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a) -> C.c_void_p:
    if a is None:
        return None
    if isinstance(a, int):
        return C.c_void_p(a)
    if hasattr(a, "data_ptr"):  # torch tensor
        return C.c_void_p(a.data_ptr())
    return a.ctypes.data_as(C.c_void_p)


def default_config(**kw) -> Config:
    cfg = Config()
    load().irr_config_default(C.byref(cfg))
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


def moldyn_params(side: float, cutoff: float) -> np.ndarray:
    """struct para {double side; double cutoffRadius;} (moldyn/moldyn.h:39-43)."""
    return np.array([side, cutoff], np.float64)


def minimd_params(cutforcesq: float, side: Optional[float] = None) -> np.ndarray:
    """double cutforcesq (miniMD/ljs.cu:123), plus the box side for the PBC map."""
    if side is None:
        return np.array([cutforcesq], np.float64)
    return np.array([cutforcesq, side], np.float64)


class DeviceEdges:
    """A device edge array owned by the library (freed on close)."""

    def __init__(self, device: int, ptr: int, count: int):
        self.device = device
        self.ptr = ptr
        self.count = count

    def to_host(self, count: Optional[int] = None) -> np.ndarray:
        """Copies the first `count` pairs (all by default) to a host array."""
        import ctypes
        cnt = self.count if count is None else max(0, min(int(count), self.count))
        out = np.empty((cnt, 2), np.int32)
        if cnt:
            cudart = _cudart()
            rc = cudart.cudaMemcpy(out.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(self.ptr),
                                   ctypes.c_size_t(out.nbytes), 2)
            if rc != 0:
                raise IrregularError(IRR_ERR_CUDA, f"cudaMemcpy failed ({rc})")
        return out

    def close(self):
        if self.ptr:
            load().irr_device_free(self.device, C.c_void_p(self.ptr))
            self.ptr = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_cudart_lib = None


def _cudart():
    global _cudart_lib
    if _cudart_lib is None:
        import ctypes.util
        for name in ("libcudart.so", "libcudart.so.13", ctypes.util.find_library("cudart")):
            if not name:
                continue
            try:
                _cudart_lib = C.CDLL(name)
                break
            except OSError:
                continue
        if _cudart_lib is None:
            raise ImportError("libcudart not found")
    return _cudart_lib


def neighbor_build(pos, box: float, list_cut2: float, device: int = 0, stream: int = 0,
                   elm_size: Optional[int] = None) -> DeviceEdges:
    """GPU half neighbour list (irr_neighbor_build); pos is a host array or a
    torch CUDA tensor of xyz records."""
    L = load()
    d_edges = C.c_void_p()
    cnt = C.c_int64()
    if hasattr(pos, "data_ptr"):
        elm = elm_size or pos.element_size() * pos.shape[-1]
        n = pos.numel() * pos.element_size() // elm
        rc = L.irr_neighbor_build(device, C.c_void_p(stream), _ptr(pos), elm, 1, n,
                                  float(box), float(list_cut2), C.byref(d_edges), C.byref(cnt))
    else:
        a = np.ascontiguousarray(pos)
        elm = elm_size or a.dtype.itemsize * a.shape[-1]
        n = a.nbytes // elm
        rc = L.irr_neighbor_build(device, C.c_void_p(stream), _ptr(a), elm, 0, n, float(box),
                                  float(list_cut2), C.byref(d_edges), C.byref(cnt))
    if rc != IRR_OK:
        raise IrregularError(rc, f"irr_neighbor_build: {L.irr_status_string(rc).decode()}")
    return DeviceEdges(device, d_edges.value or 0, cnt.value)


class Handle:
    """Owning wrapper of one irr_handle."""

    def __init__(self, cfg: Optional[Config] = None, **kw):
        L = load()
        if cfg is None:
            cfg = default_config(**kw)
        h = C.c_void_p()
        rc = L.irr_create(C.byref(cfg), C.byref(h))
        if rc != IRR_OK:
            raise IrregularError(rc, f"irr_create: {L.irr_status_string(rc).decode()}")
        self._h = h
        self.cfg = cfg

    def _check(self, rc: int, what: str):
        if rc != IRR_OK:
            msg = load().irr_last_error(self._h)
            raise IrregularError(rc, f"{what}: {msg.decode() if msg else ''}")

    @property
    def raw(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            load().irr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr: int):
        self._check(load().irr_set_stream(self._h, C.c_void_p(stream_ptr)), "irr_set_stream")

    def set_map(self, idx: int):
        self._check(load().irr_set_map(self._h, int(idx)), "irr_set_map")

    def set_reduce(self, idx: int):
        self._check(load().irr_set_reduce(self._h, int(idx)), "irr_set_reduce")

    def set_user_map(self, launch_fn: int, value_size: int, value_kind: int = 1, ctx: int = 0):
        """irr_set_user_map: bind a user map's launch function (an address,
        e.g. the irr_compat_user_launch of a library built from
        compat/irregular/irr_user_map.cu); value_kind 1 = float records."""
        self._check(load().irr_set_user_map(self._h, C.c_void_p(launch_fn), C.c_void_p(ctx),
                                            int(value_size), int(value_kind)), "irr_set_user_map")

    def set_coordinates(self, coords: np.ndarray):
        """irr_set_coordinates: (n, 2|3) float32 or float64 points that order the
        nodes of a handle with a user map."""
        a = np.ascontiguousarray(coords)
        if a.dtype not in (np.float32, np.float64) or a.ndim != 2:
            raise ValueError("coordinates: an (n, dims) float32 or float64 array")
        self._check(load().irr_set_coordinates(self._h, _ptr(a), a.dtype.itemsize, a.shape[1],
                                               a.shape[0]), "irr_set_coordinates")

    def set_params(self, blob: np.ndarray):
        blob = np.ascontiguousarray(blob)
        self._check(load().irr_set_params(self._h, _ptr(blob), blob.nbytes), "irr_set_params")

    def set_edges_device(self, d_ptr: int, num_edges: int):
        """Edges already in device memory (2 * num_edges int32 at d_ptr)."""
        self._check(load().irr_set_edges_device(self._h, C.c_void_p(d_ptr), int(num_edges)),
                    "irr_set_edges_device")

    def set_edges(self, edges):
        if isinstance(edges, DeviceEdges):
            self.set_edges_device(edges.ptr, edges.count)
            return
        if hasattr(edges, "data_ptr"):
            self._check(load().irr_set_edges_device(self._h, _ptr(edges), edges.numel() // 2),
                        "irr_set_edges_device")
            return
        e = np.ascontiguousarray(edges, np.int32).reshape(-1, 2)
        self._check(load().irr_set_edges(self._h, _ptr(e), e.shape[0]), "irr_set_edges")

    def set_nodes(self, nodes, elm_size: Optional[int] = None, n: Optional[int] = None):
        if hasattr(nodes, "data_ptr"):
            elm = elm_size or nodes.element_size() * nodes.shape[-1]
            cnt = n if n is not None else nodes.numel() * nodes.element_size() // elm
            self._check(load().irr_set_nodes_device(self._h, _ptr(nodes), elm, cnt),
                        "irr_set_nodes_device")
            return
        a = np.ascontiguousarray(nodes)
        elm = elm_size or a.dtype.itemsize * (a.shape[-1] if a.ndim > 1 else 1)
        cnt = n if n is not None else a.nbytes // elm
        self._check(load().irr_set_nodes(self._h, _ptr(a), elm, cnt), "irr_set_nodes")

    def init(self):
        self._check(load().irr_init(self._h), "irr_init")

    def step(self):
        self._check(load().irr_step(self._h), "irr_step")

    def sync(self):
        self._check(load().irr_sync(self._h), "irr_sync")

    def step_pipelined(self, nodes: np.ndarray, out: np.ndarray, node_elm: int = 12,
                       out_elm: int = 12):
        """irr_step_pipelined: upload nodes, reduce, read the result into out,
        overlapped with the neighbouring steps; out is valid after
        pipeline_sync().  Both arrays must stay alive (and nodes unchanged)
        until then."""
        self._check(load().irr_step_pipelined(self._h, _ptr(nodes), int(node_elm), _ptr(out),
                                              int(out_elm)), "irr_step_pipelined")

    def pipeline_sync(self):
        self._check(load().irr_pipeline_sync(self._h), "irr_pipeline_sync")

    def set_wait_limit(self, limit_us: int, withhold_once: bool = False):
        """irr_set_wait_limit: the device-side wait limit, and (withhold_once)
        a next step whose waits all run out, to test the time-out path."""
        self._check(load().irr_set_wait_limit(self._h, int(limit_us), int(withhold_once)),
                    "irr_set_wait_limit")

    def set_shard(self, own_lo: int, own_hi: int):
        """irr_set_shard: reduce (and return) only rows [own_lo, own_hi)."""
        self._check(load().irr_set_shard(self._h, int(own_lo), int(own_hi)), "irr_set_shard")

    def set_nodes_range(self, nodes, first: int, elm_size: Optional[int] = None):
        """irr_set_nodes_range[_device]: replace node records [first, first + len)."""
        if hasattr(nodes, "data_ptr"):
            elm = elm_size or nodes.element_size() * nodes.shape[-1]
            cnt = nodes.numel() * nodes.element_size() // elm
            self._check(load().irr_set_nodes_range_device(self._h, _ptr(nodes), elm, int(first), cnt),
                        "irr_set_nodes_range_device")
            return
        a = np.ascontiguousarray(nodes)
        elm = elm_size or a.dtype.itemsize * (a.shape[-1] if a.ndim > 1 else 1)
        self._check(load().irr_set_nodes_range(self._h, _ptr(a), elm, int(first), a.nbytes // elm),
                    "irr_set_nodes_range")

    def get_result(self, out: Optional[np.ndarray] = None, elm_size: int = 12) -> np.ndarray:
        info = self.info()
        n = info.own_hi - info.own_lo
        if out is None:
            dt = np.float64 if elm_size == 24 else np.float32
            out = np.empty((n, elm_size // np.dtype(dt).itemsize), dt)
        self._check(load().irr_get_result(self._h, _ptr(out), elm_size), "irr_get_result")
        return out

    def get_result_device(self, d_out, elm_size: int = 16):
        self._check(load().irr_get_result_device(self._h, _ptr(d_out), elm_size),
                    "irr_get_result_device")

    def info(self) -> Info:
        inf = Info()
        self._check(load().irr_get_info(self._h, C.byref(inf)), "irr_get_info")
        return inf

    def autotune(self):
        self._check(load().irr_autotune(self._h), "irr_autotune")

    def staged(self) -> dict:
        """The staged layout (irr_get_staged): items (k, 6), slice_off, words, ids."""
        return _staged_of(self)

    def partition(self, with_entries: bool = True):
        """(perm, row_off, col) of a partitioned handle; col is None when
        with_entries is False (the entries are not copied)."""
        inf = self.info()
        n, m = inf.num_nodes, inf.num_entries
        perm = np.zeros(n, np.int32)
        row_off = np.zeros(n + 1, np.int64)
        col = np.zeros(max(m, 1), np.int32) if with_entries else None
        self._check(load().irr_get_partition(self._h, _ptr(perm), _ptr(row_off),
                                             _ptr(col) if with_entries else None),
                    "irr_get_partition")
        return perm, row_off, (col[:m] if with_entries else None)


def _staged_of(handle) -> dict:
    L = load()
    counts = np.zeros(3, np.int64)
    handle._check(L.irr_get_staged(handle._h, _ptr(counts), None, None, None, None), "irr_get_staged")
    ni, nw, nd = (int(x) for x in counts)
    n = handle.info().num_nodes
    items = np.zeros((max(ni, 1), 6), np.int32)
    slice_off = np.zeros((n + 7) // 8 + 1, np.uint32)
    words = np.zeros(max(nw, 1), np.uint32)
    ids = np.zeros(max(nd, 1), np.int32)
    handle._check(L.irr_get_staged(handle._h, _ptr(counts), _ptr(items), _ptr(slice_off),
                                   _ptr(words), _ptr(ids)), "irr_get_staged")
    return {"items": items[:ni], "slice_off": slice_off, "words": words[:nw], "ids": ids[:nd]}


def read_graph(path: str, one_based: bool = False) -> np.ndarray:
    """moldyn's adjacency file -> (e, 2) int32 half list (irr_read_graph)."""
    L = load()
    n, e = C.c_int64(), C.c_int64()
    p = os.fsencode(path)
    rc = L.irr_read_graph(p, C.byref(n), C.byref(e), None, 0, int(one_based))
    if rc not in (IRR_OK,):
        raise IrregularError(rc, f"irr_read_graph({path}): {L.irr_status_string(rc).decode()}")
    out = np.zeros((e.value, 2), np.int32)
    rc = L.irr_read_graph(p, C.byref(n), C.byref(e), _ptr(out), e.value, int(one_based))
    if rc != IRR_OK:
        raise IrregularError(rc, f"irr_read_graph({path})")
    return out


def read_coords(path: str, num_nodes: int) -> np.ndarray:
    out = np.zeros((num_nodes, 3), np.float64)
    rc = load().irr_read_coords(os.fsencode(path), num_nodes, _ptr(out))
    if rc != IRR_OK:
        raise IrregularError(rc, f"irr_read_coords({path})")
    return out


def write_graph(path: str, num_nodes: int, edges) -> None:
    e = np.ascontiguousarray(edges, np.int32).reshape(-1, 2)
    rc = load().irr_write_graph(os.fsencode(path), num_nodes, _ptr(e), e.shape[0])
    if rc != IRR_OK:
        raise IrregularError(rc, f"irr_write_graph({path})")


def write_coords(path: str, xyz) -> None:
    a = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
    rc = load().irr_write_coords(os.fsencode(path), a.shape[0], _ptr(a))
    if rc != IRR_OK:
        raise IrregularError(rc, f"irr_write_coords({path})")


class Batch:
    """Many partitioned handles reduced by one persistent launch per step."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        rc = load().irr_batch_create(device, C.byref(h))
        if rc != IRR_OK:
            raise IrregularError(rc, "irr_batch_create")
        self._h = h
        self.handles = []

    def _check(self, rc, what):
        if rc != IRR_OK:
            msg = load().irr_batch_last_error(self._h)
            raise IrregularError(rc, f"{what}: {msg.decode() if msg else ''}")

    def set_stream(self, stream_ptr: int):
        self._check(load().irr_batch_set_stream(self._h, C.c_void_p(stream_ptr)), "set_stream")

    def add(self, handle: "Handle"):
        self._check(load().irr_batch_add(self._h, handle.raw), "irr_batch_add")
        self.handles.append(handle)  # keep the instance alive

    def finalize(self, autotune: bool = False):
        self._check(load().irr_batch_finalize(self._h, 1 if autotune else 0), "irr_batch_finalize")

    def capture(self):
        self._check(load().irr_batch_capture(self._h), "irr_batch_capture")

    def step(self):
        self._check(load().irr_batch_step(self._h), "irr_batch_step")

    def sync(self):
        self._check(load().irr_batch_sync(self._h), "irr_batch_sync")

    def info(self) -> BatchInfo:
        inf = BatchInfo()
        self._check(load().irr_batch_get_info(self._h, C.byref(inf)), "irr_batch_get_info")
        return inf

    def close(self):
        if getattr(self, "_h", None):
            load().irr_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def serve(**kw):
    """Runs the MD serving loop (irr_serve_run); returns (stats, jobs)."""
    L = load()
    cfg = ServeConfig()
    L.irr_serve_config_default(C.byref(cfg))
    for k, v in kw.items():
        setattr(cfg, k, v)
    stats = ServeStats()
    jobs = (ServeJob * max(cfg.num_jobs, 1))()
    rc = L.irr_serve_run(C.byref(cfg), C.byref(stats), C.cast(jobs, C.c_void_p))
    if rc != IRR_OK:
        raise IrregularError(rc, f"irr_serve_run: {L.irr_status_string(rc).decode()}")
    return stats, list(jobs)[: cfg.num_jobs]


def serve_job_state(job: int, **kw):
    """Job `job` of the stream the serve() keywords describe (irr_serve_job_state,
    host only): (atoms, side, positions (n, 3), velocities (n, 3))."""
    L = load()
    cfg = ServeConfig()
    L.irr_serve_config_default(C.byref(cfg))
    for k, v in kw.items():
        setattr(cfg, k, v)
    n, side = I64(), C.c_double()
    rc = L.irr_serve_job_state(C.byref(cfg), int(job), C.byref(n), C.byref(side), None, None)
    if rc != IRR_OK:
        raise IrregularError(rc, f"irr_serve_job_state: {L.irr_status_string(rc).decode()}")
    pos = np.zeros((n.value, 3), np.float64)
    vel = np.zeros((n.value, 3), np.float64)
    rc = L.irr_serve_job_state(C.byref(cfg), int(job), None, None, _ptr(pos), _ptr(vel))
    if rc != IRR_OK:
        raise IrregularError(rc, "irr_serve_job_state")
    return n.value, side.value, pos, vel


def serve_job_sizes(**kw):
    """Atom counts of every job of the stream the serve() keywords describe."""
    L = load()
    cfg = ServeConfig()
    L.irr_serve_config_default(C.byref(cfg))
    for k, v in kw.items():
        setattr(cfg, k, v)
    out = []
    for j in range(cfg.num_jobs):
        n = I64()
        rc = L.irr_serve_job_state(C.byref(cfg), j, C.byref(n), None, None, None)
        if rc != IRR_OK:
            raise IrregularError(rc, "irr_serve_job_state")
        out.append(n.value)
    return out


def state_digest(pos) -> int:
    """The digest irr_serve_job.state_hash reports, computed on the host: the sum
    mod 2^64, over atoms k (the caller's order) and components c, of
    mix64(bits(x_kc) + 0x9e3779b97f4a7c15 * (3k + c + 1)), mix64 being
    SplitMix64's finaliser."""
    x = np.ascontiguousarray(pos, np.float64).reshape(-1).view(np.uint64)
    k = np.arange(x.shape[0], dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15) * (k + np.uint64(1))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
        return int(z.sum(dtype=np.uint64))


class MD:
    """GPU Lennard-Jones MD (irr_md_*): FP64 state and integration, FP32 forces."""

    def __init__(self, pos, vel, side: float, dt: float = 0.005, cutforce: float = 2.5,
                 skin: float = 0.3, rebuild_every: int = 20, device: int = 0,
                 reorder_every: Optional[int] = None, exec_plain: bool = False,
                 row_slots: int = 0):
        L = load()
        cfg = MDConfig()
        L.irr_md_config_default(C.byref(cfg))
        cfg.device, cfg.dt, cfg.cutforce, cfg.skin = device, dt, cutforce, skin
        cfg.side, cfg.rebuild_every = side, rebuild_every
        if reorder_every is not None:
            cfg.reorder_every = reorder_every
        cfg.exec_plain = 1 if exec_plain else 0
        cfg.row_slots = int(row_slots)
        p = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        v = np.ascontiguousarray(vel, np.float64).reshape(-1, 3)
        self.n = p.shape[0]
        h = C.c_void_p()
        rc = L.irr_md_create(C.byref(cfg), _ptr(p), _ptr(v), self.n, C.byref(h))
        if rc != IRR_OK:
            raise IrregularError(rc, f"irr_md_create: {L.irr_status_string(rc).decode()}")
        self._h = h

    def _check(self, rc, what):
        if rc != IRR_OK:
            msg = load().irr_md_last_error(self._h)
            raise IrregularError(rc, f"{what}: {msg.decode() if msg else ''}")

    def set_stream(self, stream_ptr: int):
        self._check(load().irr_md_set_stream(self._h, C.c_void_p(stream_ptr)), "irr_md_set_stream")

    def run(self, steps: int):
        self._check(load().irr_md_run(self._h, int(steps)), "irr_md_run")

    def energy(self):
        ke, pe, vir = C.c_double(), C.c_double(), C.c_double()
        self._check(load().irr_md_energy(self._h, C.byref(ke), C.byref(pe), C.byref(vir)),
                    "irr_md_energy")
        return ke.value, pe.value, vir.value

    def state(self):
        p = np.empty((self.n, 3), np.float64)
        v = np.empty((self.n, 3), np.float64)
        self._check(load().irr_md_get_state(self._h, _ptr(p), _ptr(v)), "irr_md_get_state")
        return p, v

    def forces(self):
        f = np.empty((self.n, 3), np.float64)
        self._check(load().irr_md_get_forces(self._h, _ptr(f)), "irr_md_get_forces")
        return f

    def info(self) -> MDInfo:
        inf = MDInfo()
        self._check(load().irr_md_get_info(self._h, C.byref(inf)), "irr_md_get_info")
        return inf

    def close(self):
        if getattr(self, "_h", None):
            load().irr_md_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class IrregularRuntime:
    """The reference's IrregularRuntime interface over the C ABI.

    Constructor arguments follow irregular_runtime.h:71-86; `num_procs`,
    `num_iters` and the edge data are accepted for source compatibility (one
    GPU, no MPI split).  `map_idx` picks a built-in user function (IRR_MAP_*);
    `user_launch` (the address of an irr_user_launch_fn, e.g. the
    irr_compat_user_launch of a library built from compat/irregular/
    irr_user_map.cu with the application's irregular.h) binds the
    application's own map and reduce tables instead, with `value_size`-byte
    results, and then `node_coordinates` ((n, node_num_dims) floats or
    doubles) order the nodes."""

    def __init__(self, num_edges, num_nodes, edges, edge_data, node_data, edge_data_elm_size,
                 node_data_elm_size, reduction_elm_size, node_num_dims=3,
                 node_coordinates=None, coordinate_size=8, parameter=None, parameter_size=None,
                 num_procs=1, num_iters=1, map_idx=IRR_MAP_LJ_MOLDYN,
                 exec_mode=IRR_EXEC_PARTITIONED, user_launch=None, value_size=12, value_kind=1,
                 **cfg_kw):
        self.num_edges = int(num_edges)
        self.num_nodes = int(num_nodes)
        self.node_elm = int(node_data_elm_size)
        self.red_elm = int(reduction_elm_size)
        self.user = user_launch is not None
        if self.user:
            self.h = Handle(default_config(exec=exec_mode, **cfg_kw))
            self.h.set_user_map(user_launch, value_size, value_kind)
            if map_idx:
                self.h.set_map(map_idx)
            if node_coordinates is not None:
                dt = np.float64 if int(coordinate_size) == 8 else np.float32
                self.h.set_coordinates(np.asarray(node_coordinates, dt).reshape(self.num_nodes, int(node_num_dims)))
        else:
            self.h = Handle(default_config(map_idx=map_idx, exec=exec_mode, **cfg_kw))
        self.h.set_params(np.ascontiguousarray(parameter))
        self.h.set_edges(np.asarray(edges, np.int32).reshape(-1, 2)[: self.num_edges])
        self.h.set_nodes(node_data, self.node_elm, self.num_nodes)

    def set_map_idx(self, idx: int):
        self.h.set_map(idx)

    def set_reduce_idx(self, idx: int):
        self.h.set_reduce(idx)

    def IrregularInit(self):
        self.h.init()

    def IrregularStart(self):
        self.h.step()

    def IrregularBarrier(self):
        self.h.sync()

    def reset_node_data(self, node_data):
        self.h.set_nodes(node_data, self.node_elm, self.num_nodes)

    def get_reduction_result(self, buffer: Optional[np.ndarray] = None) -> np.ndarray:
        return self.h.get_result(buffer, self.red_elm)
