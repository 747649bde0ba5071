"""Drop-in: the reference's own drivers compile and link unchanged against the
compat headers (ipdps15-pattern_gb300/compat) and the C-ABI library (CPU).

Runs only where the reference tree is present.  Each driver source is fed to
the compiler on stdin so that its quoted includes of the runtime headers
resolve to the compat directory, not to the reference's runtime beside it;
the drivers' own headers and support files come from the reference tree.
"""
import os
import subprocess

import pytest

from conftest import PKG, ROOT
from oracle.oracle import reference_tree

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


def link(objs, out):
    r = subprocess.run(["g++", "-o", out] + objs + ["-L", PKG, "-lirregular_gb300",
                                                     f"-Wl,-rpath,{PKG}", "-lm", "-fopenmp"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    undefined = subprocess.run(["nm", "-u", out], capture_output=True, text=True).stdout
    return undefined


def test_moldyn_driver_compiles_and_links_unchanged(built_lib, tmp_path):
    d = os.path.join(REF, "moldyn")
    objs = [compile_from_stdin(os.path.join(d, "moldyn.cu"), str(tmp_path / "moldyn.o"), d),
            compile_from_stdin(os.path.join(d, "misc.c"), str(tmp_path / "misc.o"), d, "c"),
            compile_from_stdin(os.path.join(d, "timer.c"), str(tmp_path / "timer.o"), d, "c")]
    und = link(objs, str(tmp_path / "moldyn"))
    for sym in ("irr_create", "irr_step", "irr_get_result", "irr_set_nodes"):
        assert sym in und


def test_minimd_driver_compiles_and_links_unchanged(built_lib, tmp_path):
    d = os.path.join(REF, "miniMD")
    objs = []
    for f in ("ljs.cu", "atom.cpp", "neighbor.cpp", "force.cpp", "setup.cpp", "thermo.cpp",
              "input.cpp"):
        objs.append(compile_from_stdin(os.path.join(d, f), str(tmp_path / (f + ".o")), d))
    objs.append(compile_from_stdin(os.path.join(d, "timer.c"), str(tmp_path / "timer.o"), d, "c"))
    und = link(objs, str(tmp_path / "miniMD"))
    assert "irr_step" in und and "irr_init" in und
