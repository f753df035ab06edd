"""Parity at the configurations' stated sizes.

  brine4352   4096 SPC/E + 128 Na+ + 128 Cl- (12544 sites), cutoff 10 A,
              alpha 0.31/A, |n| <= 12 (3576 k-vectors)
  drude32768  32768 Drude waters (98304 sites + 32768 shells), cutoff 12 A,
              alpha 0.26/A, |n| <= 20 (16700 k-vectors), ASPC k=2 + one SCF
              iteration per step

On a relaxed configuration of each: the FP64 device forces and energies
against the threaded oracle (1e-10 of the force scale; the oracle is pinned
to cook's dumps at the fixture sizes); the mixed path against FP64 within
the 1e-5 relative force RMS bound, with its energies and the k-space energy
bias of the tensor-core Ewald passes (their FP32 accumulation rounds toward
zero) stated; a few MD steps of both precisions stay together."""
import os

import numpy as np
import pytest

import macsimus_gb300 as M
from macsimus_gb300 import configs
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-5


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


@pytest.fixture(scope="module", params=["brine4352", "drude32768"])
def relaxed(request):
    w = configs.workload(request.param, seed=5)
    return configs.equilibrate(w, steps=100, polar_steps=40)


def paths(w):
    args = (w["system"], [w["L"]] * 3, w["cutoff"], w["alpha"], w["kappa"])
    kw = dict(h=w["h"], epsc=1e-10, aspc_k=w["aspc_k"], scf_iter=w["scf_iter"])
    return M.ForcePath(*args, precision="mixed", **kw), M.ForcePath(*args, precision="fp64", **kw)


def test_fullsize_fp64_matches_oracle_and_mixed_matches_fp64(relaxed):
    w = relaxed
    fm_path, fd_path = paths(w)
    assert fd_path.nkvec == {"brine4352": 3576, "drude32768": 16700}[w["name"]]
    fm, em = fm_path.forces(w["r"], measure=True)
    fd, ed = fd_path.forces(w["r"], measure=True)
    orc = O.Oracle(w["system"], [w["L"]] * 3, w["cutoff"], w["alpha"], w["kappa"])
    fo, eo = orc.forces(w["r"], nthreads=os.cpu_count() or 4)
    # FP64 device = oracle
    assert rel_rms(fd, fo) < 1e-10
    for k in ("el", "er", "ek"):
        assert abs(ed[k] - eo[k]) <= 1e-10 * abs(eo["eself"]), k
    assert abs(ed["lj"] - eo["lj"]) <= 1e-10 * abs(eo["lj"])
    # mixed within the bound of FP64; energies on the Ewald energy scale
    err = rel_rms(fm, fd)
    bias = (em["ek"] - ed["ek"]) / abs(ed["ek"])
    print("%s: mixed force rel RMS %.2e, k-space energy (mixed - FP64)/|FP64| %.2e, "
          "el %.2e of |E_self|, lj %.2e" % (w["name"], err, bias,
                                            (em["el"] - ed["el"]) / abs(ed["eself"]),
                                            (em["lj"] - ed["lj"]) / abs(ed["lj"])))
    assert err < MIXED_TOL
    for k in ("el", "er", "ek"):
        assert abs(em[k] - ed[k]) <= 2e-6 * abs(ed["eself"]), k
    assert abs(em["lj"] - ed["lj"]) <= 1e-5 * abs(ed["lj"])
    assert abs(bias) < 1e-5


def test_fullsize_md_steps_agree(relaxed):
    """three MD steps (Drude: ASPC + one SCF iteration + SHAKE each) from the
    same state in both precisions"""
    w = relaxed
    ns = w["system"].ns
    out = {}
    for name, p in zip(("mixed", "fp64"), paths(w)):
        p.md_set_state(w["r"], w["r1"])
        en = p.md_steps(3)
        out[name] = (p.md_get_state()[0], en)
    dr = np.abs(out["mixed"][0] - out["fp64"][0])
    assert dr[:ns].max() < 1e-5
    if w["system"].polar:
        assert dr[ns:].max() < 1e-5
    em, ed = out["mixed"][1], out["fp64"][1]
    assert abs(em["ekin"] - ed["ekin"]) < 1e-6 * ed["ekin"]
    # the pressure tensor of the measured step: its virial part carries the
    # mixed rounding of the electrostatic terms, which is relative to the
    # Ewald energy scale |E_self| (2e-6 of it, as the energies above)
    V = w["L"] ** 3
    assert np.abs(np.array(em["Ptens"]) - np.array(ed["Ptens"])).max() < \
        1e-5 * np.abs(ed["Pkin"]).max() + 2e-6 * abs(ed["eself"]) / V
