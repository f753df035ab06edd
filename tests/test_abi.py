"""The C-ABI library loads and exports every entry point of include/macgpu.h
(no GPU needed: nothing is called that touches a device)."""
import os
import re
import subprocess

import pytest

from macsimus_gb300 import build as B

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    txt = open(os.path.join(REPO, "include", "macgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mg_[a-z_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib_path():
    return B.build()


def test_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True,
                         text=True, check=True).stdout
    exported = set(l.split()[-1] for l in out.splitlines() if l.strip())
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing
    assert len(declared_functions()) >= 12


def test_library_loads_without_device(lib_path):
    import macsimus_gb300 as M
    L = M.library()
    for f in declared_functions():
        assert hasattr(L, f)


def test_product_does_not_reference_oracle():
    """the product package never imports or links the oracle"""
    for root, _, files in os.walk(os.path.join(REPO, "macsimus_gb300")):
        for fn in files:
            if fn.endswith((".py", ".cu", ".cpp", ".h")):
                src = open(os.path.join(root, fn)).read()
                assert "cookoracle" not in src and "from oracle" not in src, fn


@pytest.mark.parametrize("cname,pyname", [
    ("mg_topology", "Topology"), ("mg_params", "Params"), ("mg_energy", "Energy"),
    ("mg_probe", "Probe"), ("mg_widom_result", "WidomResult"),
    ("mg_adjoint_out", "AdjointOut")])
def test_ctypes_layout_matches_header(cname, pyname, tmp_path):
    """the Python mirror's structs have the header's size and field offsets
    (a C program built with the host compiler prints them)"""
    import ctypes
    import macsimus_gb300 as M
    cls = getattr(M, pyname)
    fields = [f[0] for f in cls._fields_]
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "macgpu.h"', 'int main(void){',
           'printf("%%zu\\n", sizeof(%s));' % cname]
    src += ['printf("%%zu\\n", offsetof(%s, %s));' % (cname, f) for f in fields]
    src.append('return 0;}')
    c = tmp_path / "layout.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), str(c), "-o", str(exe)],
                   check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    assert out[0] == ctypes.sizeof(cls)
    assert out[1:] == [getattr(cls, f).offset for f in fields]
