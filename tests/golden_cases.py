"""Loading of the golden fixtures written by tests/golden/make_golden.py."""
import json
import os

import numpy as np

from macsimus_gb300 import forcefield as ff

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["spce216", "brine532", "spce864", "widom500", "tip4p216"]
POLAR_CASES = ["drude216"]


def load(case):
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    meta = json.load(open(os.path.join(GOLDEN, case + ".json")))
    p = meta["params"]
    system = ff.build_system(p["species"], p["N"])
    ewald = dict(L=np.array(g["L"]), cutoff=p["cutoff"], alpha=p["alpha"],
                 kappa=(p["kn"] + 1e-6) / p["L"])
    return g, meta, system, ewald
