"""Device thermostats (cook's Berendsen and Bussi, sim/thermo.c) against the
oracle's step + factor, and their long-run temperatures."""
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
