"""NVE energy conservation of the device integrator against cook's own.

tests/golden/nve864.json holds the per-step Etot that cook printed for the
864-water SPC/E box (L = 29.65 A, cutoff 12 A, alpha 0.26/A, |n| <= 8,
h = 2 fs, SHAKE 1e-10): 1500 Berendsen steps (tau.T 0.1 ps) from its crystal
start, then 5000 NVE steps.  The device runs the same protocol from cook's
crystal start (the first two force evaluations of tests/golden/spce864) in
both precisions.  Trajectories are chaotic, so the comparison is by
statistics of Etot(t) over the NVE part: the drift (slope of a line through
block means, with its standard error), the fluctuation about that line and
the mean step-to-step change.
"""
import json
import os

import numpy as np
import pytest

import macsimus_gb300 as M
from golden_cases import GOLDEN, load

pytestmark = pytest.mark.gpu


def drift(t, E, nblock=10):
    """slope of the block means of E(t) and its standard error; the noise
    of means over blocks of hundreds of steps is nearly independent"""
    t, E = np.asarray(t), np.asarray(E)
    n = len(E) // nblock * nblock
    tb = t[:n].reshape(nblock, -1).mean(1)
    Eb = E[:n].reshape(nblock, -1).mean(1)
    x = tb - tb.mean()
    s = (x * (Eb - Eb.mean())).sum() / (x * x).sum()
    res = Eb - Eb.mean() - s * x
    se = np.sqrt((res * res).sum() / (nblock - 2) / (x * x).sum())
    return s, se


def fluctuation(t, E):
    t, E = np.asarray(t), np.asarray(E)
    p = np.polyfit(t - t.mean(), E, 1)
    return float(np.std(E - np.polyval(p, t - t.mean())))


def device_run(precision, nequil, nrun):
    g, meta, system, ew = load("spce864")
    h = meta["params"]["h"]
    kw = dict(precision=precision, h=h, epsc=1e-10, omegac=meta["omegac"])
    eq = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"],
                     thermostat="berendsen", T=298.0, tau_T=0.1, **kw)
    eq.md_set_state(g["r"][1], g["r"][1] - g["r"][0])
    eq.md_steps(nequil, measure=False)
    r, r1 = eq.md_get_state()
    del eq
    fp = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"], **kw)
    fp.md_set_state(r, r1)
    nf = 3 * system.ns - len(system.cons_len) - 3
    E, T = [], []
    for _ in range(nrun):
        en = fp.md_steps(1)
        E.append(en["el"] + en["lj"] + en["ekin"])
        T.append(2 * en["ekin"] / nf)
    return np.arange(1, nrun + 1) * h, np.array(E), np.array(T)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nve_drift_no_worse_than_reference(precision):
    ref = json.load(open(os.path.join(GOLDEN, "nve864.json")))
    Ec = np.array(ref["Etot"])
    tc = ref["t0"] + ref["params"]["h"] * np.arange(len(Ec))
    nequil = ref["params"]["sweeps"][0]["steps"] - 1
    t, E, T = device_run(precision, nequil, len(Ec))
    sc, sec = drift(tc, Ec)
    sg, seg = drift(t, E)
    fc, fg = fluctuation(tc, Ec), fluctuation(t, E)
    dc, dg = np.abs(np.diff(Ec)).mean(), np.abs(np.diff(E)).mean()
    print("cook: drift %.1f +- %.1f K/ps, fluctuation %.1f K, |dE| %.1f K; "
          "%s: drift %.1f +- %.1f K/ps, fluctuation %.1f K, |dE| %.1f K, T %.1f K"
          % (sc, sec, fc, dc, precision, sg, seg, fg, dg, T.mean()))
    # the same equilibrium
    assert abs(T.mean() / np.mean(ref["Tkin"]) - 1) < 0.03
    # drift: within three standard errors of cook's magnitude
    assert abs(sg) <= abs(sc) + 3 * np.hypot(sec, seg), (sg, seg, sc, sec)
    # fluctuation and step-to-step changes of Etot: cook's size
    assert fg < 1.3 * fc, (fg, fc)
    assert dg < 1.3 * dc, (dg, dc)


def ensemble_drifts(runs_E, h_block):
    """per run the drift (K/ps) of block means, then their mean and the
    standard error of that mean over the runs"""
    s = []
    for E in runs_E:
        E = np.asarray(E)
        t = (np.arange(len(E)) + 0.5) * h_block
        x = t - t.mean()
        s.append(float((x * (E - E.mean())).sum() / (x * x).sum()))
    s = np.array(s)
    return s, s.mean(), s.std(ddof=1) / np.sqrt(len(s))


def device_ensemble(precision, ref):
    """the same protocol as cook's four runs: 864 SPC/E from lattice starts
    with independent seeds, Berendsen 0.1 ps for the equilibration steps,
    then NVE; Etot of every step in block means"""
    from macsimus_gb300 import configs
    p = ref["params"]
    g, meta, system, ew = load("spce864")
    out = []
    for seed in p["seeds"]:
        w = configs.workload("spce864", seed=seed)
        kw = dict(precision=precision, h=p["h"], epsc=p["epsc"], omegac=meta["omegac"])
        eq = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"],
                         thermostat="berendsen", T=298.0, tau_T=0.1, **kw)
        eq.md_set_state(w["r"], w["r1"])
        eq.md_steps(p["equil"], measure=False)
        r, r1 = eq.md_get_state()
        eq.close()
        fp = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"], **kw)
        fp.md_set_state(r, r1)
        E = np.empty(p["steps"])
        for k in range(p["steps"]):
            en = fp.md_steps(1)
            E[k] = en["el"] + en["lj"] + en["ekin"]
        fp.close()
        nb = p["steps"] // p["block"]
        out.append(E[:nb * p["block"]].reshape(nb, p["block"]).mean(1))
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nve_drift_ensemble_against_reference(precision):
    """four independent 50 ps NVE runs on each side (tests/golden/nve864x4:
    cook's own runs from crystal starts with seeds 11..14, 1500 Berendsen
    steps then 25000 NVE steps): the mean drift of the device is at most
    1.2 x the magnitude of cook's plus two combined standard errors (the
    standard errors from the spread of the four runs)"""
    ref = json.load(open(os.path.join(GOLDEN, "nve864x4.json")))
    p = ref["params"]
    hb = p["h"] * p["block"]
    sc, mc, ec = ensemble_drifts([r["Etot_block"] for r in ref["runs"]], hb)
    runs = device_ensemble(precision, ref)
    sg, mg, eg = ensemble_drifts(runs, hb)
    print("NVE drift over 4 x %d steps, K/ps: cook %s -> %.2f +- %.2f; %s %s -> %.2f +- %.2f"
          % (p["steps"], np.round(sc, 2), mc, ec, precision, np.round(sg, 2), mg, eg))
    # the same equilibrium temperature
    assert abs(np.mean([r["Tkin_mean"] for r in ref["runs"]]) / 298.0 - 1) < 0.03
    assert abs(mg) <= 1.2 * abs(mc) + 2 * np.hypot(ec, eg), (mg, eg, mc, ec)
