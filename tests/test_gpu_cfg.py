"""Resume parity through cook's .cfg files on the device: the state cook
saved (tests/golden/resume216_a.cfg), loaded into a context and advanced,
gives cook's own continuation (run B); the same with r1 halved gives the
continuation cook made from the file that macsimus_gb300.cfgfile wrote
(run C); and a state saved by the device reads back unchanged and resumes
exactly as the uninterrupted run."""
import os

import numpy as np
import pytest

import macsimus_gb300 as M
from macsimus_gb300 import cfgfile as cf
from test_cfgfile import A, fixture

pytestmark = pytest.mark.gpu


def context(precision, meta, system, ew, omegac):
    p = meta["params"]
    return M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"],
                       precision=precision, h=p["h"], epsc=p["epsc"], omegac=omegac)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 1e-6)])
@pytest.mark.parametrize("run", ["B", "C"])
def test_device_resumes_from_cook_cfg(precision, tol, run):
    meta, g, system, ew, omegac = fixture()
    fp = context(precision, meta, system, ew, omegac)
    c = fp.md_load_cfg(A)
    if run == "C":
        r, r1 = cf.state_from_cfg(c, system.ns)
        fp.md_set_state(r, r1 * meta["params"]["r1_scale"])
    fp.md_steps(meta["params"]["steps_b"], measure=False)
    r, r1 = fp.md_get_state()
    assert np.abs(r - g["r" + run]).max() < tol
    assert np.abs(r1 - g["r1" + run]).max() < tol


def test_saved_state_reads_back_and_resumes(tmp_path):
    meta, g, system, ew, omegac = fixture()
    fp = context("fp64", meta, system, ew, omegac)
    c = fp.md_load_cfg(A)
    fp.md_steps(2, measure=False)
    path = str(tmp_path / "saved.cfg")
    fp.md_save_cfg(path, c, t=c["t"] + 2 * c["h"])
    r, r1 = fp.md_get_state()
    # the same state copied into caller-owned buffers
    bufs = (np.empty(r.size), np.empty(r1.size))
    fp.md_get_state(out=bufs)
    assert np.array_equal(bufs[0].reshape(-1, 3), r) and np.array_equal(bufs[1].reshape(-1, 3), r1)
    with pytest.raises(ValueError):
        fp.md_get_state(out=(np.empty(5), np.empty(5)))
    back = cf.read_cfg(path)
    rb, r1b = cf.state_from_cfg(back, system.ns)
    assert np.array_equal(rb, r) and np.array_equal(r1b, r1)
    assert abs(back["t"] - (c["t"] + 2 * c["h"])) < 1e-15
    fp.md_steps(2, measure=False)
    fp2 = context("fp64", meta, system, ew, omegac)
    fp2.md_load_cfg(path)
    fp2.md_steps(2, measure=False)
    assert np.array_equal(fp2.md_get_state()[0], fp.md_get_state()[0])


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-8), ("mixed", 1e-5)])
def test_drude_device_resumes_from_cook_cfg(precision, tol):
    """a Drude context loaded from cook's POLAR .cfg (sites and Drude
    displacements; the ASPC history restarted from cfg[0] and cfg[1] as cook
    restarts it) continues as cook continued the same file"""
    import json
    from golden_cases import GOLDEN
    from macsimus_gb300 import forcefield as ff
    meta = json.load(open(os.path.join(GOLDEN, "resume_drude216.json")))
    g = np.load(os.path.join(GOLDEN, "resume_drude216.npz"))
    p = meta["params"]
    system = ff.build_system(p["species"], p["N"])
    omegac = json.load(open(os.path.join(GOLDEN, "drude216.json")))["omegac"]
    fp = M.ForcePath(system, np.array([p["L"]] * 3), p["cutoff"], p["alpha"],
                     (p["kn"] + 1e-6) / p["L"], precision=precision, h=p["h"], epsc=p["epsc"],
                     omegac=omegac, aspc_k=2, scf_iter=1)
    fp.md_load_cfg(os.path.join(GOLDEN, "resume_drude216_a.cfg"))
    fp.md_steps(p["steps_b"], measure=False)
    r, _ = fp.md_get_state()
    ns = system.ns
    assert np.abs(r[:ns] - g["rB"][:ns]).max() < tol
    assert np.abs(r[ns:] - g["rB"][ns:]).max() < tol
