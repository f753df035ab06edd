"""The oracle's pressure against cook's printed pressure tensor.

Fixtures tests/golden/press_*.json (tests/golden/make_golden.py): cook built
with PRESSURETENSOR 7 continues its own .cfg state by one measured step and
prints, with 9 significant digits, the virial, kinetic and total pressure
tensors (measurePconstraints, sim/constrd.c:115-265: the force virial plus
the SHAKE constraint virial of sim/virc.c divided by h^2, the VERLET=3
kinetic tensor of sim/shakev3.c), the constraint pressure Pvirc, the scalar
virial En.vir and the pressure Pevir.  The oracle repeats that step: forces
(+ the Drude SCF iteration, + the dependants' force redistribution with
the virial terms of the out-of-plane kinds) and
leap-frog + SHAKE with the measured sums."""
import numpy as np
import pytest

from golden_cases import PRESSURE_CASES, PT_NAMES, load_pressure
from oracle import oracle as O

# printed 9 significant digits; each tensor is compared on the scale of its
# largest component (the total tensor on the scale of its kinetic part: it
# is the sum of large parts of opposite sign), scalars relative to themselves
DIGITS = 5e-9


def oracle_step(case):
    meta, g, system, ew, r, r1 = load_pressure(case)
    p = meta["params"]
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    om = meta["omegac"] / 2
    if getattr(system, "polar", False):
        _, _, press = O.drude_md(orc, system, r, r1, p["h"], 2, 1, 1, p["epsc"], meta["omegac"],
                                 measure=True)
        return meta, g, system, press, orc, r
    if system.ndep:
        r = O.depend_r(system, r)
    f, en = orc.forces(r, measure=True, nthreads=4)
    if system.ndep:
        f, dvir, dpvir = O.depend_f(system, f, r, virial=True)
        en = dict(en, vir=en["vir"] + dvir, Pvir=np.asarray(en["Pvir"]) + dpvir)
    meas = np.zeros(13)
    _, _, it, ek = orc.shake_step(r, r1, f, p["h"], eps=p["epsc"], omega=om, meas=meas)
    press = O.measure_pressure(en, meas, ek, orc.L)
    press["ekin"] = ek
    return meta, g, system, press, orc, r


def check_against_cook(press, stats, L, tol=DIGITS, scalar_tol=None, whole_scale=False):
    """press: K/A^3 values (Pvir, Pkin, Ptens, P), virc and vir in K.
    whole_scale: every tensor on the scale of the pressure's two parts,
    max |Pvir| + max |Pkin| (a rounding error of FP32 forces is relative to
    the virial, not to what remains of it in the sum)"""
    scalar_tol = tol if scalar_tol is None else scalar_tol
    V = float(np.prod(L))
    U = O.PUNIT
    kin = np.abs(np.array([stats["Pkin.%s [Pa]" % n] for n in PT_NAMES])).max()
    vir = np.abs(np.array([stats["Pvir.%s [Pa]" % n] for n in PT_NAMES])).max()
    for part in ("Pvir", "Pkin", "Ptens"):
        ref = np.array([stats["%s.%s [Pa]" % (part, n)] for n in PT_NAMES])
        scale = max(np.abs(ref).max(), kin if part == "Ptens" else 0)
        if whole_scale:
            scale = vir + kin
        assert np.abs(np.asarray(press[part]) * U - ref).max() < tol * scale, part
    # the constraint pressure En.virc Punit / (3 V), En.vir after the
    # constraint and electrostatic parts, and Pevir
    assert abs(press["virc"] * U / 3 / V / stats["Pvirc [Pa]"] - 1) < scalar_tol
    assert abs(press["vir"] / stats["virial"] - 1) < scalar_tol
    assert abs(press["P"] * U / stats["Pevir [Pa]"] - 1) < scalar_tol


@pytest.mark.parametrize("case", PRESSURE_CASES)
def test_oracle_pressure_matches_cook(case):
    meta, g, system, press, orc, r = oracle_step(case)
    # the oracle starts from the state cook dumped its forces for
    assert np.abs(r[:system.ns] - g["r"]).max() < 1e-9
    check_against_cook(press, meta["stats"], orc.L)
    # kinetic temperature 2 Ekin / No.f, No.f = 3 (ns - ndep) - nc - 3
    nf = 3 * (system.ns - system.ndep) - len(system.cons) - 3
    assert abs(2 * press["ekin"] / nf / meta["stats"]["Tkin"] - 1) < DIGITS
