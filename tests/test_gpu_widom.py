"""Widom insertions on the GPU (through the C ABI) against the oracle on the
same insertion stream: per-insertion energies and the Boltzmann sum, both
precisions; a multi-site charged ghost (SPC/E water into SPC/E water)."""
import numpy as np
import pytest

import macsimus_gb300 as M
from golden_cases import load
from macsimus_gb300 import forcefield as ff
from oracle import oracle as O

pytestmark = pytest.mark.gpu

PRB = [ff.TYPE_ORDER.index("PRB")]
T = 298.0


def ctx(case, precision, **kw):
    g, meta, system, ew = load(case)
    fp = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"],
                     precision=precision, **kw)
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    return g, meta, system, ew, fp, orc


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("cells", [1, 2])
def test_lj_probe_energies_and_average(precision, cells):
    g, meta, system, ew, fp, orc = ctx("widom500", precision, cells_per_cutoff=cells)
    r = g["r"][-1]
    fp.forces(r)
    n = 40000
    res = fp.widom(PRB, n=n, seed=4242, T=T, energies=True)
    s, corr, Uo = orc.widom(r, PRB, [0.0], [0, 0, 0], n, 4242, T, energies=True)
    U = res["U"]
    ok = Uo < 50 * T
    if precision == "fp64":
        assert np.abs(U[ok] - Uo[ok]).max() < 1e-9 * (np.abs(Uo[ok]).max() + 1)
        assert abs(res["sum"] - s) <= 1e-11 * s
    else:
        # FP32 pair energies: ~1e-6 of the largest terms of the sum
        assert np.abs(U[ok] - Uo[ok]).max() < 1e-2 + 1e-6 * np.abs(Uo[ok]).max()
        assert abs(res["sum"] - s) <= 2e-6 * s
    assert abs(res["corr"] - corr) <= 1e-10 * abs(corr)
    V = float(np.prod(ew["L"]))
    assert abs(res["factor"] - np.exp(-corr / (V * T))) < 1e-14
    assert abs(res["mu"] + T * np.log(s / n * res["factor"])) < (1e-8 if precision == "fp64" else 1e-3)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_water_ghost_into_water(precision):
    """a rigid SPC/E ghost (3 charged sites, random orientations) into the
    864-water box"""
    g, meta, system, ew, fp, orc = ctx("spce864", precision)
    r = g["r"][0]
    fp.forces(r)
    sp = ff.spce()
    types = [ff.TYPE_ORDER.index(t) for t in sp.sites]
    q = np.array(sp.charges) * ff.ELECTRON
    geo = sp.geometry - sp.geometry[0]
    n = 8000
    res = fp.widom(types, geometry=geo, charges=q, n=n, seed=77, T=T, energies=True)
    s, corr, Uo = orc.widom(r, types, q, geo, n, 77, T, energies=True)
    # insertions without a core overlap (a water ghost rarely finds a cavity)
    ok = Uo < 1e5
    assert ok.sum() > 100
    err = np.abs(res["U"][ok] - Uo[ok])
    if precision == "fp64":
        assert (err <= 1e-9 * (np.abs(Uo[ok]) + 1e3)).all()
    else:
        assert (err <= 1e-5 * (np.abs(Uo[ok]) + 1e4)).all()
    assert abs(res["sum"] - s) <= (1e-10 if precision == "fp64" else 1e-4) * s + 1e-300


def test_reproducible_and_uses_last_force_configuration():
    g, meta, system, ew, fp, orc = ctx("widom500", "mixed", h=0.002)
    r0 = g["r"][-1]
    fp.forces(r0)
    a = fp.widom(PRB, n=20000, seed=3, T=T)
    b = fp.widom(PRB, n=20000, seed=3, T=T)
    assert a["sum"] == b["sum"]
    # after one MD step the last force evaluation was at the starting point
    fp.md_set_state(r0, np.zeros_like(r0))
    fp.md_steps(1, measure=False)
    c = fp.widom(PRB, n=20000, seed=3, T=T)
    assert abs(c["sum"] - a["sum"]) <= 1e-12 * a["sum"]


def test_errors_are_reported():
    g, meta, system, ew = load("widom500")
    fp = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    with pytest.raises(M.MGError):
        fp.widom(PRB, n=10)          # no force evaluation yet
    fp.forces(g["r"][-1])
    with pytest.raises(M.MGError):
        fp.widom([99], n=10)         # type out of range
    gd, md, sd, ed = load("drude216")
    fd = M.ForcePath(sd, ed["L"], ed["cutoff"], ed["alpha"], ed["kappa"])
    fd.forces(np.vstack([gd["r"][0], gd["rD"][0]]))
    with pytest.raises(M.MGError):
        fd.widom([0], n=10)          # Drude systems are not supported


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_identity_change_vs_oracle_and_reference(precision):
    """cook's XWidom on the device: every AP cation of the last configuration
    changed into APV; energy changes per molecule against the oracle and the
    chemical potential against cook's printed value (6 digits)"""
    g, meta, system, ew = load("xwidom500")
    T = 298.0
    fp = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"],
                     precision=precision)
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    r = g["r"][-1]
    fp.forces(r)
    ap = list(range(system.counts[0]))
    vt, vq = [ff.TYPE_ORDER.index("APV")], [0.8 * ff.ELECTRON]
    res = fp.xwidom(ap, vt, vq, T, energies=True)
    s, dU = orc.xwidom(r, ap, vt, vq, T)
    tol = 1e-7 if precision == "fp64" else 2e-3          # K
    assert np.abs(res["dU"] - dU).max() < tol * max(1.0, np.abs(dU).max())
    assert abs(res["sum"] / s - 1) < (1e-9 if precision == "fp64" else 1e-5)
    mu = meta["xwidom"]["mu_raw_K"]
    assert abs(res["mu"] - mu) <= 6e-6 * abs(mu) + (0 if precision == "fp64" else 0.01)
