"""The compat IrregularRuntime class at run time (GPU): a C++ driver making
moldyn's call sequence, built here against the compat headers with the
built-in moldyn law (IRR_COMPAT_MAP), must reproduce the reference's own
result (golden fixture) within the FP32 tolerance."""
import os
import subprocess

import numpy as np
import pytest

from conftest import PKG, ROOT
from helpers import TOL_VS_REFERENCE, load_golden, oracle_param, scaled_error

pytestmark = pytest.mark.gpu


def build_driver(tmp_path):
    exe = str(tmp_path / "moldyn_like")
    src = os.path.join(ROOT, "tests", "drop_in", "moldyn_like.cpp")
    # the library's built-in moldyn law (the fast path); test_gpu_plugin.py
    # runs the same driver with the map from an application table
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-DIRR_COMPAT_MAP=IRR_MAP_LJ_MOLDYN", "-I",
                        os.path.join(PKG, "compat"), "-I",
                        os.path.join(ROOT, "include"), src, "-o", exe, "-L", PKG,
                        "-lirregular_gb300", f"-Wl,-rpath,{PKG}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("name", ["moldyn_random_2048", "moldyn_shuffled_dups_1500"])
def test_compat_runtime_matches_reference(built_lib, oracle_lib, tmp_path, name):
    O = oracle_lib
    c = load_golden(name)
    exe = build_driver(tmp_path)
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
