"""The C-ABI library loads and exports every symbol include/*.h declares
(CPU only: no compute call is made without a GPU)."""
import glob
import os
import re
import subprocess

import pytest

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        names |= set(re.findall(r"IRR_API\s+[\w\s\*]*?\b(irr_\w+)\s*\(", src))
    return names


def exported_symbols(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if " T " in ln}


def test_header_declares_entry_points():
    names = declared_symbols()
    for required in ("irr_create", "irr_destroy", "irr_set_edges", "irr_set_nodes",
                     "irr_set_params", "irr_step", "irr_get_result", "irr_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(built_lib):
    import irregular_gb300 as irr
    exported = exported_symbols(irr.LIB_PATH)
    declared = declared_symbols()
    assert declared <= exported, f"missing: {sorted(declared - exported)}"
    assert {s for s in exported if s.startswith("irr_")} == declared


def test_binding_covers_header(built_lib):
    import irregular_gb300 as irr
    assert declared_symbols() <= set(irr._SIGS)


def test_status_strings_and_defaults(built_lib):
    import irregular_gb300 as irr
    L = irr.load()
    assert L.irr_status_string(0) == b"ok"
    assert L.irr_status_string(2) == b"edge endpoint out of range"
    cfg = irr.default_config()
    assert cfg.exec == irr.IRR_EXEC_PARTITIONED and cfg.reorder == 1 and cfg.stage_smem == -1


def test_serve_and_md_config_defaults_and_validation(built_lib):
    """New fields sit in the configs' reserved space with their defaults, and
    a bad admission policy, serving mode, MD force path or slot count is
    refused before any device call."""
    import ctypes as C
    import irregular_gb300 as irr
    L = irr.load()
    sc = irr.ServeConfig()
    L.irr_serve_config_default(C.byref(sc))
    assert sc.policy == irr.IRR_SERVE_FIFO and sc.max_resident == 64
    mc = irr.MDConfig()
    L.irr_md_config_default(C.byref(mc))
    assert mc.reorder_every == 10 and mc.rebuild_every == 20 and mc.exec_plain == 0 and mc.row_slots == 0
    # the sizes the structs had before the new fields took reserved slots
    assert C.sizeof(irr.ServeConfig) == 144 and C.sizeof(irr.MDConfig) == 72
    for bad in (dict(policy=7), dict(mode=9)):
        with pytest.raises(irr.IrregularError) as ei:
            irr.serve(**bad)
        assert ei.value.status == irr.IRR_ERR_ARG
    # an MD force path other than 0 (partitioned) or 1 (plain)
    import numpy as np
    mc.side, mc.exec_plain = 10.0, 7
    pos = np.zeros((4, 3))
    h = C.c_void_p()
    rc = L.irr_md_create(C.byref(mc), pos.ctypes.data_as(C.c_void_p), pos.ctypes.data_as(C.c_void_p),
                         4, C.byref(h))
    assert rc == irr.IRR_ERR_ARG and not h.value
    mc.exec_plain, mc.row_slots = 0, 5000
    rc = L.irr_md_create(C.byref(mc), pos.ctypes.data_as(C.c_void_p), pos.ctypes.data_as(C.c_void_p),
                         4, C.byref(h))
    assert rc == irr.IRR_ERR_ARG and not h.value


def test_create_rejects_bad_config_without_crashing(built_lib):
    import irregular_gb300 as irr
    for bad in (dict(exec=7), dict(map_idx=9), dict(block_nodes=100), dict(lanes_per_row=3), dict(lanes_per_row=64)):
        with pytest.raises(irr.IrregularError) as ei:
            irr.Handle(irr.default_config(**bad))
        assert ei.value.status in (irr.IRR_ERR_ARG, irr.IRR_ERR_CUDA)


def test_no_gpu_fails_loudly(built_lib):
    """On a host without a GPU the product path raises; it never computes on the CPU."""
    import irregular_gb300 as irr
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(irr.IrregularError) as ei:
        irr.Handle()
    assert ei.value.status == irr.IRR_ERR_CUDA
