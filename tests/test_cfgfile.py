"""cook's .cfg configuration files (macsimus_gb300.cfgfile) against files
that the reference cook wrote and read.

Fixture tests/golden/resume216 (tests/golden/make_golden.py): cook run A
from its crystal start (216 SPC/E, 4 steps) wrote resume216_a.cfg; run B
continued from that file for 3 steps; run C continued for 3 steps from a
file that cfgfile.write_cfg made from A's state with r1 halved.  The final
cfg[0] (positions) and cfg[1] (r(t) - r(t-h)) of B and C are stored.
"""
import hashlib
import json
import os
import struct

import numpy as np
import pytest

from golden_cases import GOLDEN
from macsimus_gb300 import cfgfile as cf
from macsimus_gb300 import forcefield as ff
from oracle import oracle as O

A = os.path.join(GOLDEN, "resume216_a.cfg")


def fixture():
    meta = json.load(open(os.path.join(GOLDEN, "resume216.json")))
    g = np.load(os.path.join(GOLDEN, "resume216.npz"))
    p = meta["params"]
    system = ff.build_system(p["species"], p["N"])
    ew = dict(L=np.array([p["L"]] * 3), cutoff=p["cutoff"], alpha=p["alpha"],
              kappa=(p["kn"] + 1e-6) / p["L"])
    # SHAKE over-relaxation of the same box (cook optimises omegac per run;
    # at epsc = 1e-10 the result does not depend on it beyond 1e-10 A)
    omegac = json.load(open(os.path.join(GOLDEN, "spce216.json")))["omegac"]
    return meta, g, system, ew, omegac


def test_reads_cook_file_and_writes_it_back_byte_for_byte(tmp_path):
    c = cf.read_cfg(A)
    assert c["cfgkey"] == 1 and not c["polar"]
    assert c["species"] == [(216, 3)] and c["N"] == 216 and c["ns"] == 648
    assert np.allclose(c["L"], 18.6206) and c["h"] == 0.002
    assert abs(c["t"] - 4 * 0.002) < 1e-12
    assert len(c["cfg"]) == 2
    r, r1 = cf.state_from_cfg(c, 648)
    assert r.shape == (648, 3) and np.all(np.isfinite(r))
    # lambda of cfg[0] is log(L) once cook derived it, else 0 (sim/simglob.h:309)
    lam = c["cfg"][0]["lam"]
    assert np.allclose(lam, 0) or np.allclose(lam, np.log(18.6206))
    # r1 = r(t) - r(t-h): a few hundredths of an angstrom per step
    assert 1e-4 < np.abs(r1).max() < 0.2
    out = tmp_path / "rt.cfg"
    cf.write_cfg(out, c)
    assert out.read_bytes() == open(A, "rb").read()


def test_writer_made_the_file_cook_continued_from():
    meta, g, system, ew, omegac = fixture()
    c = cf.read_cfg(A)
    r, r1 = cf.state_from_cfg(c, system.ns)
    w = cf.cfg_with_state(c, r, r1 * meta["params"]["r1_scale"])
    path = os.path.join(os.environ.get("TMPDIR", "/tmp"), "mg_cfg_written_%d.cfg" % os.getpid())
    try:
        cf.write_cfg(path, w)
        assert hashlib.sha256(open(path, "rb").read()).hexdigest() == meta["sha256_written"]
        back = cf.read_cfg(path)
        assert np.array_equal(back["cfg"][1]["rp"], r1 * meta["params"]["r1_scale"])
    finally:
        if os.path.exists(path):
            os.remove(path)


@pytest.mark.parametrize("run", ["B", "C"])
def test_oracle_resumes_where_cook_resumed(run):
    """the state read from the file, advanced by the oracle's forces + SHAKE
    + normalize for the same number of steps, is cook's final state"""
    meta, g, system, ew, omegac = fixture()
    p = meta["params"]
    r, r1 = cf.state_from_cfg(cf.read_cfg(A), system.ns)
    if run == "C":
        r1 = r1 * p["r1_scale"]
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    for _ in range(p["steps_b"]):
        f, _ = orc.forces(r, measure=False, nthreads=4)
        r, r1, it, _ = orc.shake_step(r, r1, f, p["h"], eps=p["epsc"], omega=omegac / 2)
        r = O.normalize(system, r, ew["L"])
    assert np.abs(r - g["r" + run]).max() < 1e-9
    assert np.abs(r1 - g["r1" + run]).max() < 1e-9


def test_damaged_files_are_refused(tmp_path):
    raw = bytearray(open(A, "rb").read())
    bad = tmp_path / "bad.cfg"
    # a flipped data byte breaks the record checksum
    raw2 = bytearray(raw)
    raw2[200] ^= 0x40
    bad.write_bytes(bytes(raw2))
    with pytest.raises(cf.CfgError):
        cf.read_cfg(bad)
    # a truncated file
    bad.write_bytes(bytes(raw[:1000]))
    with pytest.raises(cf.CfgError):
        cf.read_cfg(bad)
    # a record size that does not match the configuration header
    raw3 = bytearray(raw)
    off = len(raw3) - 8 - 15616 - 4
    struct.pack_into("<i", raw3, off + 4, 12345)
    bad.write_bytes(bytes(raw3))
    with pytest.raises(cf.CfgError):
        cf.read_cfg(bad)
    # a state of the wrong shape
    with pytest.raises(cf.CfgError):
        cf.cfg_with_state(cf.read_cfg(A), np.zeros((10, 3)), np.zeros((10, 3)))


def test_polar_cfg_holds_the_drude_half():
    """cook's Drude build (POLAR, cfgkey 3) saves 2 ns vectors per
    configuration, the Drude displacements after the sites, and tau.dip as
    key 17 (sim/simils.c:1505-1509); the file round-trips byte for byte"""
    path = os.path.join(GOLDEN, "resume_drude216_a.cfg")
    c = cf.read_cfg(path)
    assert c["cfgkey"] == 3 and c["polar"] and 17 in c["keys"]
    r, r1 = cf.state_from_cfg(c, 648)
    assert r.shape == (1296, 3) and r1.shape == (1296, 3)
    # Drude displacements: a few hundredths of an angstrom
    assert 1e-3 < np.abs(r[648:]).max() < 0.2
    out = os.path.join(os.environ.get("TMPDIR", "/tmp"), "mg_cfg_polar_%d.cfg" % os.getpid())
    try:
        cf.write_cfg(out, c)
        assert open(out, "rb").read() == open(path, "rb").read()
    finally:
        if os.path.exists(out):
            os.remove(out)
