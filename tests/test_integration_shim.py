"""The cook shim written out in INTEGRATION.md compiles against cook's own
headers.

The block under "The shim cook would compile" flattens cook's tables
(spec[], molec[], sitedef[], the dependant lists) into mg_topology and
replaces forces() (cook/forces.c:93); the next block is the measured MD
step (what measurePconstraints assembles), the third the replacement of
Widom() (sim/simmeas.c:1821).  gcc checks them in syntax-only mode with the
compile-time switches of the cook builds made by oracle/build_ref.sh:
Ewald + linked cells (cookew), its Drude form (cookpol), the pressure-
tensor build (cookewpt, with the measured step) and the Widom build
(cookwidom, with the Widom replacement).  The reference sources are
needed; without them (or without the recipe's per-build simopt.h) the test
skips."""
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


def shim_blocks():
    text = open(os.path.join(REPO, "INTEGRATION.md")).read()
    i = text.index("## The shim cook would compile")
    blocks = re.findall(r"```c\n(.*?)```", text[i:], re.S)
    assert len(blocks) >= 3, "the shim, the measured step and Widom"
    return blocks[:3]


def unit(build):
    """the C source checked for one build: the shim, plus the fragment
    that build enables"""
    shim, md, widom = shim_blocks()
    if build == "cookewpt":
        return shim + "\nvoid gpu_md_measured(int noint)\n{\n  int i;\n" + md + "}\n"
    if build == "cookwidom":
        return shim + "\n" + widom
    return shim


@pytest.mark.parametrize("build", ["cookew", "cookpol", "cookewpt", "cookwidom"])
def test_integration_shim_compiles_against_cook(build, tmp_path):
    ref = reference_dir()
    if ref is None or shutil.which("gcc") is None:
        pytest.skip("reference sources or gcc not available")
    opt = os.path.join(REFBIN, build + ".d")
    if not os.path.exists(os.path.join(opt, "simopt.h")):
        pytest.skip("oracle/build_ref.sh has not configured %s" % build)
    src = tmp_path / "forces_gpu.c"
    src.write_text(unit(build))
    cmd = ["gcc", "-fsyntax-only", "-DSCR", "-Werror=implicit-function-declaration",
           "-Werror=incompatible-pointer-types", "-Werror=int-conversion", "-I" + opt]
    cmd += ["-I" + os.path.join(ref, d) for d in ("gen", "sim", "sim/lj", "cook")]
    cmd += ["-I" + os.path.join(REPO, "include"), str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_integration_shim_covers_the_boundary():
    """the shim passes every kind of dependant, takes the inputs cook keeps
    local, and replaces forces() with cook's signature"""
    shim = shim_blocks()[0]
    assert "dep_type" in shim and "dep_par" in shim
    assert "gpu_forces_init(double LJcutoff, int comb_rule)" in shim
    assert "void forces(ToIntPtr B, ToIntPtr A)" in shim
    assert "double Widom(int sp, int ncyc, double corr)" in shim_blocks()[2]
