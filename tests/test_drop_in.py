"""Drop-in: the reference's own drivers compile and link unchanged against the
compat headers (ipdps15-pattern_gb300/compat) and the C-ABI library (CPU),
with their own irregular.h compiled into the user-map plugin
(compat/irregular/irr_user_map.cu), as the reference compiles it into its
executors.

Runs only where the reference tree is present.  Each driver source is fed to
the compiler on stdin so that its quoted includes of the runtime headers
resolve to the compat directory, not to the reference's runtime beside it;
the drivers' own headers and support files come from the reference tree.
"""
import os
import shutil
import subprocess

import pytest

from conftest import PKG, ROOT
from oracle.oracle import reference_tree
from plugin_build import build_plugins

REF = reference_tree()
COMPAT = os.path.join(PKG, "compat")

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "moldyn", "irregular")),
                                reason="reference tree not present")


def compile_from_stdin(src, out, inc, lang="c++", std="-std=c++17"):
    cmd = (["g++", std, "-x", "c++"] if lang == "c++" else ["gcc", "-x", "c"])
    cmd += ["-O1", "-w", "-I", COMPAT, "-I", os.path.join(ROOT, "include"), "-I", inc, "-c", "-",
            "-o", out]
    with open(src) as f:
        r = subprocess.run(cmd, stdin=f, capture_output=True, text=True)
    assert r.returncode == 0, f"{os.path.basename(src)}:\n{r.stderr[-2000:]}"
    return out


def user_map_object(driver_dir, tmp_path):
    """The driver's irregular.h through the plugin shim (see
    test_plugin_build.py for why the application directory is a copy)."""
    app = tmp_path / "app"
    app.mkdir()
    for f in ("irregular.h", "moldyn.h"):
        shutil.copy(os.path.join(driver_dir, f), app / f)
    obj = str(tmp_path / "user_map.o")
    build_plugins({"user_map": (str(app), obj, False, (), True)})
    return obj


def link(objs, out):
    cuda_lib = "/usr/local/cuda/lib64"
    r = subprocess.run(["g++", "-o", out] + objs + ["-L", PKG, "-lirregular_gb300",
                                                     f"-Wl,-rpath,{PKG}", "-L", cuda_lib, "-lcudart",
                                                     f"-Wl,-rpath,{cuda_lib}", "-lm", "-fopenmp"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    undefined = subprocess.run(["nm", "-u", out], capture_output=True, text=True).stdout
    return undefined


def test_moldyn_driver_compiles_and_links_unchanged(built_lib, tmp_path):
    d = os.path.join(REF, "moldyn")
    objs = [compile_from_stdin(os.path.join(d, "moldyn.cu"), str(tmp_path / "moldyn.o"), d),
            compile_from_stdin(os.path.join(d, "misc.c"), str(tmp_path / "misc.o"), d, "c"),
            compile_from_stdin(os.path.join(d, "timer.c"), str(tmp_path / "timer.o"), d, "c"),
            user_map_object(d, tmp_path)]
    und = link(objs, str(tmp_path / "moldyn"))
    for sym in ("irr_create", "irr_step", "irr_get_result", "irr_set_nodes", "irr_set_user_map",
                "irr_set_coordinates"):
        assert sym in und


def test_minimd_driver_compiles_and_links_unchanged(built_lib, tmp_path):
    d = os.path.join(REF, "miniMD")
    objs = []
    for f in ("ljs.cu", "atom.cpp", "neighbor.cpp", "force.cpp", "setup.cpp", "thermo.cpp",
              "input.cpp"):
        objs.append(compile_from_stdin(os.path.join(d, f), str(tmp_path / (f + ".o")), d))
    objs.append(compile_from_stdin(os.path.join(d, "timer.c"), str(tmp_path / "timer.o"), d, "c"))
    objs.append(user_map_object(d, tmp_path))
    und = link(objs, str(tmp_path / "miniMD"))
    assert "irr_step" in und and "irr_init" in und and "irr_set_user_map" in und


def test_driver_without_a_map_does_not_link(built_lib, tmp_path):
    """Neither IRR_COMPAT_MAP nor the plugin object: the link fails on the
    registration symbol instead of running some built-in law."""
    d = os.path.join(REF, "moldyn")
    objs = [compile_from_stdin(os.path.join(d, "moldyn.cu"), str(tmp_path / "moldyn.o"), d),
            compile_from_stdin(os.path.join(d, "misc.c"), str(tmp_path / "misc.o"), d, "c"),
            compile_from_stdin(os.path.join(d, "timer.c"), str(tmp_path / "timer.o"), d, "c")]
    r = subprocess.run(["g++", "-o", str(tmp_path / "moldyn")] + objs +
                       ["-L", PKG, "-lirregular_gb300", f"-Wl,-rpath,{PKG}", "-lm", "-fopenmp"],
                       capture_output=True, text=True)
    assert r.returncode != 0 and "irr_compat_register_user_map" in r.stderr
