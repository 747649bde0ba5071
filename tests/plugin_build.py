"""Builds user-map plugins: compat/irregular/irr_user_map.cu compiled against
an application directory that holds an irregular.h (the tests' fixtures under
tests/plugin/, or a copy of a reference driver's), for sm_103a."""
from __future__ import annotations

import os
import shutil
import subprocess

from conftest import PKG, ROOT

COMPAT = os.path.join(PKG, "compat")
USER_MAP_TU = os.path.join(COMPAT, "irregular", "irr_user_map.cu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def plugin_cmd(app_dir: str, out: str, shared: bool, defines=(), fmad: bool = True) -> list:
    cmd = [nvcc()] + ARCH + ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", app_dir, "-I", COMPAT,
                             "-I", os.path.join(ROOT, "include")]
    cmd += [f"-D{d}" for d in defines]
    if not fmad:
        cmd += ["-fmad=false"]
    if shared:
        cmd += ["-shared", "-cudart", "shared", USER_MAP_TU, "-o", out, "-L", PKG, "-lirregular_gb300",
                f"-Xlinker=-rpath,{PKG}"]
    else:
        cmd += ["-c", USER_MAP_TU, "-o", out]
    return cmd


def build_plugins(jobs: dict) -> dict:
    """jobs: name -> (app_dir, out, shared, defines, fmad); compiled in
    parallel.  Returns name -> out; raises with the compiler's output."""
    procs = {name: subprocess.Popen(plugin_cmd(*args), stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                                    text=True)
             for name, args in jobs.items()}
    outs = {}
    for name, p in procs.items():
        log, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"plugin {name} failed to build:\n{log[-3000:]}")
        outs[name] = jobs[name][1]
    return outs
