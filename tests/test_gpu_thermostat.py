"""Device thermostats (cook's Berendsen, Bussi and Nose-Hoover, sim/thermo.c)
against the oracle's step + factor and cook's Nose-Hoover trajectory, and
their long-run temperatures."""
import numpy as np
import pytest

import macsimus_gb300 as M
from golden_cases import load
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def fp_for(meta, system, ew, precision, **kw):
    return M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"],
                       precision=precision, h=meta["params"]["h"], epsc=meta["params"]["epsc"],
                       omegac=meta["omegac"], **kw)


@pytest.mark.parametrize("kind", [1, 2])
def test_one_thermostatted_step_matches_oracle(kind):
    g, meta, system, ew = load("spce216")
    h = meta["params"]["h"]
    r, r1 = g["r"][2], g["r"][2] - g["r"][1]
    nf = 3 * system.ns - len(system.cons_len) - 3
    fp = fp_for(meta, system, ew, "fp64", thermostat=kind, T=298.0, tau_T=0.05, seed=11)
    fp.md_set_state(r, r1)
    fp.md_steps(1, measure=False)
    rg, r1g = fp.md_get_state()
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    f, _ = orc.forces(r, measure=False, nthreads=4)
    ro, r1o, it, ekin = orc.shake_step(r, r1, f, h, eps=meta["params"]["epsc"],
                                      omega=meta["omegac"] / 2)
    # the oracle's ekin is sum m (V1^2 + V2^2) / (4 h^2)
    z = O.thermostat_factor(kind, ekin * 4 * h * h, h, nf, 298.0, 0.05, 11, 0)
    assert abs(fp.thermostat_factor() - z) < 1e-12
    assert np.abs(rg - ro).max() < 1e-9
    assert np.abs(r1g - r1o * z).max() < 1e-9 * np.abs(r1o).max()


@pytest.mark.parametrize("kind", [1, 2])
def test_thermostat_holds_the_temperature(kind):
    g, meta, system, ew = load("spce864")
    h = meta["params"]["h"]
    nf = 3 * system.ns - len(system.cons_len) - 3
    fp = fp_for(meta, system, ew, "mixed", thermostat=kind, T=298.0, tau_T=0.05, seed=3)
    # the lattice start releases potential energy for a while; the
    # thermostat carries it away, then holds 298 K
    fp.md_set_state(g["r"][1], g["r"][1] - g["r"][0])
    fp.md_steps(600, measure=False)
    temps = []
    for _ in range(40):
        en = fp.md_steps(5)
        temps.append(2 * en["ekin"] / nf)
    late = np.mean(temps)
    assert abs(late / 298.0 - 1) < 0.03, (late, temps[:5])


def test_bussi_stream_is_reproducible():
    g, meta, system, ew = load("spce216")
    out = []
    for _ in range(2):
        fp = fp_for(meta, system, ew, "mixed", thermostat=2, T=298.0, tau_T=0.1, seed=99)
        fp.md_set_state(g["r"][2], g["r"][2] - g["r"][1])
        fp.md_steps(20, measure=False)
        out.append(fp.md_get_state()[1])
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("precision,tol", [("fp64", 5e-8), ("mixed", 2e-5)])
def test_nose_hoover_matches_reference_trajectory(precision, tol):
    """cook's Nose-Hoover Verlet+SHAKE (thermostat=2 in cook, tau.T 0.05 ps,
    TRVP k -> 2) on the device: five steps from the state of cook's second
    dump reproduce cook's dumped positions (FP64: the dumps' 12 printed
    decimals; mixed: the force error times h^2/m) and the oracle's
    thermostat variables"""
    g, meta, system, ew = load("nose216")
    h = meta["params"]["h"]
    nf = 3 * system.ns - len(system.cons_len) - 3
    r = g["r"][1].copy()
    r1 = g["vlb_r"][0].astype(np.float64) * h
    fp = fp_for(meta, system, ew, precision, thermostat="nose", T=298.0, tau_T=0.05)
    fp.md_set_state(r, r1)
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    nh = O.NoseHoover(298.0, 0.05, nf, h)
    ro, r1o = r, r1
    for step in range(5):
        en = fp.md_steps(1)
        f, _ = orc.forces(ro, measure=False, nthreads=4)
        ro, r1o, it, ek = nh.step(orc, ro, r1o, f, omega=meta["omegac"] / 2)
        rg, r1g = fp.md_get_state()
        if step + 2 < g["r"].shape[0]:
            assert np.abs(rg - g["r"][step + 2]).max() < tol, step
        assert np.abs(rg - ro).max() < tol, step
        logs, logsv, ext = fp.nose_state()
        assert abs(logsv - nh.logsv) < 1e-6 * abs(nh.logsv) + (1e-12 if precision == "fp64"
                                                               else 1e-9), step
        assert abs(logs - nh.logs) < 1e-6 * abs(nh.logs) + 1e-9, step
    assert abs(en["ekin"] / meta["Ekin_last"] - 1) < (1e-8 if precision == "fp64" else 1e-5)
    assert abs(ext - nh.ext) < 1e-5 * abs(nh.ext) + 1e-3


def test_nose_hoover_holds_the_temperature_and_conserves_its_energy():
    """Nose-Hoover NVT from the 864-water lattice start: the temperature
    relaxes to 298 K, and the extended energy Etot + Eext of cook's VERLET=3
    form fluctuates far less than Etot itself while the thermostat moves
    energy in and out"""
    g, meta, system, ew = load("spce864")
    nf = 3 * system.ns - len(system.cons_len) - 3
    fp = fp_for(meta, system, ew, "mixed", thermostat="nose", T=298.0, tau_T=0.1)
    fp.md_set_state(g["r"][1], g["r"][1] - g["r"][0])
    fp.md_steps(1500, measure=False)
    temps, ham, cons = [], [], []
    for _ in range(100):
        en = fp.md_steps(10)
        ext = fp.nose_state()[2]
        temps.append(2 * en["ekin"] / nf)
        ham.append(en["el"] + en["lj"] + en["ekin"])
        cons.append(ham[-1] + ext)
    assert abs(np.mean(temps) / 298.0 - 1) < 0.03, temps[:5]
    assert np.std(cons) < 0.2 * np.std(ham), (np.std(cons), np.std(ham))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bounddr_and_drift_removal_match_reference_trajectory(precision):
    """the device steps with drmax = 0.02 A and the momentum drift removed
    after every step reproduce cook's run with drmax = -0.02 (tests/golden/
    bounddr216); the limiter reports the sites it reduced"""
    from golden_cases import load
    g, meta, system, ew = load("bounddr216")
    p = meta["params"]
    fp = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"],
                     precision=precision, h=p["h"], epsc=p["epsc"], omegac=meta["omegac"],
                     drmax=p["drmax"], drift_step=True)
    R = g["r"]
    r1, _, _ = O.bounddr(R[2] - R[1], p["drmax"])
    r1, _ = O.remove_drift(system, r1)
    fp.md_set_state(R[2], r1)
    tol = 1e-9 if precision == "fp64" else 1e-6
    nred = 0
    for k in range(2):
        fp.md_steps(1, measure=False)
        r, r1d = fp.md_get_state()
        assert np.abs(r - R[3 + k]).max() < tol
        n, q = fp.bounddr_report()
        _, no, qo = O.bounddr(r - R[2 + k], p["drmax"])
        assert n == no and abs(q - qo) < 1e-6
        nred += n
        assert np.abs((system.mass[:, None] * r1d).sum(0)).max() < 1e-9 * system.mass.sum()
    assert nred > 100


def test_remove_drift_matches_oracle():
    from golden_cases import load
    g, meta, system, ew = load("spce216")
    fp = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"], precision="fp64")
    r1 = (g["r"][2] - g["r"][1]) + np.array([1e-3, -2e-3, 5e-4])
    fp.md_set_state(g["r"][2], r1)
    v = fp.remove_drift()
    _, r1d = fp.md_get_state()
    r1o, vo = O.remove_drift(system, r1)
    assert np.abs(r1d - r1o).max() < 1e-15
    assert np.abs(v - vo / meta["params"]["h"]).max() < 1e-12
