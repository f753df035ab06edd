"""The cook shim written out in INTEGRATION.md compiles against cook's own
headers.

The block under "The shim cook would compile" flattens cook's tables
(spec[], molec[], sitedef[], the dependant lists) into mg_topology and
replaces forces() (cook/forces.c:93).  gcc checks it in syntax-only mode
with the compile-time switches of two cook builds made by
oracle/build_ref.sh: Ewald + linked cells (cookew) and its Drude form
(cookpol).  The reference sources are needed; without them (or without the
recipe's per-build simopt.h) the test skips."""
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
REFBIN = os.path.join(REPO, "oracle", "_ref")


def reference_dir():
    p = os.path.join(REFBIN, "REFERENCE_DIR")
    if not os.path.exists(p):
        return None
    d = open(p).read().strip()
    return d if os.path.isdir(os.path.join(d, "cook")) else None


def shim_source():
    text = open(os.path.join(REPO, "INTEGRATION.md")).read()
    i = text.index("## The shim cook would compile")
    m = re.search(r"```c\n(.*?)```", text[i:], re.S)
    assert m, "no C block under the shim heading"
    return m.group(1)


@pytest.mark.parametrize("build", ["cookew", "cookpol"])
def test_integration_shim_compiles_against_cook(build, tmp_path):
    ref = reference_dir()
    if ref is None or shutil.which("gcc") is None:
        pytest.skip("reference sources or gcc not available")
    opt = os.path.join(REFBIN, build + ".d")
    if not os.path.exists(os.path.join(opt, "simopt.h")):
        pytest.skip("oracle/build_ref.sh has not configured %s" % build)
    src = tmp_path / "forces_gpu.c"
    src.write_text(shim_source())
    cmd = ["gcc", "-fsyntax-only", "-DSCR", "-Werror=implicit-function-declaration",
           "-Werror=incompatible-pointer-types", "-Werror=int-conversion", "-I" + opt]
    cmd += ["-I" + os.path.join(ref, d) for d in ("gen", "sim", "sim/lj", "cook")]
    cmd += ["-I" + os.path.join(REPO, "include"), str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    # the shim passes every kind of dependant, and the inputs cook keeps local
    text = shim_source()
    assert "dep_type" in text and "dep_par" in text
    assert "gpu_forces_init(double LJcutoff, int comb_rule)" in text
