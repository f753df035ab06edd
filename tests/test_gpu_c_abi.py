"""A plain C program (tests/c/spce_abi.c, compiled here with gcc and linked
against libmacgpu.so) builds the SPC/E topology from arrays as a cook shim
would and calls mg_create -> mg_forces -> mg_md_set_state -> mg_md_steps ->
mg_md_get_state -> mg_destroy on the 216-water fixture: its forces equal
cook's dump, its step cook's next positions."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import macsimus_gb300 as M
from golden_cases import load

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = M.library()._name
    out = str(tmp_path_factory.mktemp("cabi") / "spce_abi")
    subprocess.run([cc, "-O2", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(REPO, "include"),
                    os.path.join(HERE, "c", "spce_abi.c"), lib, "-lm",
                    "-Wl,-rpath," + os.path.dirname(lib), "-o", out], check=True)
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_plain_c_caller(program, tmp_path, precision):
    g, meta, system, ew = load("spce216")
    p = meta["params"]
    R = g["r"]
    head = [system.nmol, ew["L"][0], ew["cutoff"], ew["alpha"], ew["kappa"], p["h"], p["epsc"],
            meta["omegac"], precision]
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    np.concatenate([np.array(head, np.float64), R[0].reshape(-1), R[2].reshape(-1),
                    (R[2] - R[1]).reshape(-1)]).tofile(fin)
    r = subprocess.run([program, fin, fout], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = np.fromfile(fout, np.float64)
    n3 = 3 * system.ns
    f, el, lj, rn = out[:n3].reshape(-1, 3), out[n3], out[n3 + 1], out[n3 + 2:].reshape(-1, 3)
    tol = 2e-10 if precision == 0 else 1e-5
    assert rel_rms(f, g["f"][0]) < tol
    assert np.abs(rn - R[3]).max() < (1e-9 if precision == 0 else 1e-6)
    # the same energies as the Python mirror of the ABI on the same context
    fp = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"],
                     precision="fp64" if precision == 0 else "mixed")
    _, en = fp.forces(R[0], measure=True)
    assert abs(el - en["el"]) < 1e-9 * abs(en["eself"]) and abs(lj - en["lj"]) < 1e-9 * abs(lj)
