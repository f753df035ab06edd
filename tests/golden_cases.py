"""Loading of the golden fixtures written by tests/golden/make_golden.py."""
import json
import os

import numpy as np

from macsimus_gb300 import forcefield as ff

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["spce216", "brine532", "spce864", "widom500", "tip4p216", "t5r216"]
POLAR_CASES = ["drude216"]


def load(case):
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    meta = json.load(open(os.path.join(GOLDEN, case + ".json")))
    p = meta["params"]
    system = ff.build_system(p["species"], p["N"])
    ewald = dict(L=np.array(g["L"]), cutoff=p["cutoff"], alpha=p["alpha"],
                 kappa=(p["kn"] + 1e-6) / p["L"], epsinf=p.get("epsinf", 3e33),
                 elcorr=p.get("elcorr", 0))
    return g, meta, system, ewald


# the dipole term of Ewald(2): finite epsinf, Yeh-Berkowitz along z, and its
# energy-only form
DIPOLE_CASES = ["dip216eps", "dip216yb", "dip216yb8"]


PRESSURE_CASES = ["press_spce216", "press_tip4p216", "press_drude216", "press_t5r216"]


def load_pressure(case):
    """cook's state (its .cfg file written after the run-A steps), the
    statistics cook printed for the one measured step that followed it
    (meta["stats"], Pa and K), the forces dumped at that state, the system
    and its Ewald parameters"""
    from macsimus_gb300 import cfgfile
    meta = json.load(open(os.path.join(GOLDEN, case + ".json")))
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    p = meta["params"]
    system = ff.build_system(p["species"], p["N"])
    c = cfgfile.read_cfg(os.path.join(GOLDEN, case + "_a.cfg"))
    r, r1 = cfgfile.state_from_cfg(c, system.ns)
    ewald = dict(L=np.array([p["L"]] * 3), cutoff=p["cutoff"], alpha=p["alpha"],
                 kappa=(p["kn"] + 1e-6) / p["L"])
    return meta, g, system, ewald, r, r1


# the printed pressure-tensor components (xx yy zz yz zx xy)
PT_NAMES = ("xx", "yy", "zz", "yz", "zx", "xy")
