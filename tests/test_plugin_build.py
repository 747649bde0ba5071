"""The irregular.h plugin boundary on CPU: user per-edge functions written in
the reference's irregular.h form compile through the compat shim
(compat/irregular/{parameters,ros}.h, irr_user_map.cu, include/
irregular_plugin.cuh) and export the launch and registration functions --
the tests' own fixtures always, and the reference's own moldyn/irregular.h and
miniMD/irregular.h (moldyn/irregular.h:9-118, miniMD/irregular.h:9-175)
wherever the reference tree is present."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT
from oracle.oracle import reference_tree
from plugin_build import build_plugins

REF = reference_tree()
FIXTURES = os.path.join(ROOT, "tests", "plugin")
EXPORTS = ("irr_compat_user_launch", "irr_compat_register_user_map")


def defined_symbols(obj):
    out = subprocess.run(["nm", obj], capture_output=True, text=True).stdout
    return {line.split()[-1] for line in out.splitlines() if " T " in line}


def test_fixture_plugins_compile(tmp_path):
    jobs = {
        "spring": (os.path.join(FIXTURES, "spring"), str(tmp_path / "spring.o"), False, (), True),
        "spring_comp": (os.path.join(FIXTURES, "spring"), str(tmp_path / "spring_comp.o"), False,
                        ("IRR_PLUGIN_COMPENSATED",), True),
        "lj": (os.path.join(FIXTURES, "lj"), str(tmp_path / "lj.o"), False, (), False),
        "lj_inline": (os.path.join(FIXTURES, "lj"), str(tmp_path / "lj_inline.o"), False,
                      ("IRR_PLUGIN_INLINE_MAP=lj_box", "IRR_PLUGIN_COMPENSATED"), True),
    }
    for name, obj in build_plugins(jobs).items():
        syms = defined_symbols(obj)
        for s in EXPORTS:
            assert s in syms, (name, s)


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "moldyn", "irregular")),
                    reason="reference tree not present")
@pytest.mark.parametrize("driver", ["moldyn", "miniMD"])
def test_reference_irregular_h_compiles_through_the_shim(tmp_path, driver):
    # The application directory for the shim: the driver's irregular.h and the
    # header it includes, without the reference runtime's irregular/
    # subdirectory (whose quoted includes would otherwise win).
    app = tmp_path / "app"
    app.mkdir()
    for f in ("irregular.h", "moldyn.h"):
        shutil.copy(os.path.join(REF, driver, f), app / f)
    obj = str(tmp_path / "user_map.o")
    build_plugins({driver: (str(app), obj, False, (), True)})
    syms = defined_symbols(obj)
    for s in EXPORTS:
        assert s in syms
