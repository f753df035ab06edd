"""The device pressure tensor against cook's printed values.

mg_md_steps fills, for the last step, the constraint virial (the SHAKE
factors of every sweep, sim/virc.c), the kinetic tensor of the leap-frog
velocities (sim/shakev3.c) and the total tensor cook's measurePconstraints
assembles (sim/constrd.c:115-265).  Each context continues cook's own .cfg
state (tests/golden/press_*_a.cfg) by the one measured step cook printed
(PRESSURETENSOR 7 build): FP64 to cook's 9 printed digits, the mixed path to
1e-5 of the pressure's scale max |Pvir| + max |Pkin|."""
import os

import numpy as np
import pytest

import macsimus_gb300 as M

from golden_cases import GOLDEN, PRESSURE_CASES, load_pressure
from test_oracle_pressure import DIGITS, check_against_cook

pytestmark = pytest.mark.gpu


def device_step(case, precision):
    meta, g, system, ew, r, r1 = load_pressure(case)
    p = meta["params"]
    kw = dict(aspc_k=2, scf_iter=1) if getattr(system, "polar", False) else {}
    fp = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"],
                     precision=precision, h=p["h"], epsc=p["epsc"], omegac=meta["omegac"], **kw)
    fp.md_load_cfg(os.path.join(GOLDEN, case + "_a.cfg"))
    en = fp.md_steps(1)
    press = dict(Pvir=(np.array(en["Ptens"]) - np.array(en["Pkin"])), Pkin=en["Pkin"],
                 Ptens=en["Ptens"], P=en["P"], virc=en["virc"],
                 vir=en["vir"] + en["virc"] + en["el"] - 2 * en["self"])
    return meta, press, ew["L"]


@pytest.mark.parametrize("case", PRESSURE_CASES)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_device_pressure_matches_cook(case, precision):
    meta, press, L = device_step(case, precision)
    if precision == "fp64":
        check_against_cook(press, meta["stats"], L, tol=DIGITS)
    else:
        check_against_cook(press, meta["stats"], L, tol=1e-5, scalar_tol=1e-5, whole_scale=True)
