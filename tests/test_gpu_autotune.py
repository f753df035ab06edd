"""The autotuner (mg_autotune) returns a valid cell subdivision and pass-1
split, and the tuned path gives the same forces."""
import numpy as np
import pytest

import macsimus_gb300 as M
from golden_cases import load

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_autotune_choice_and_forces(precision):
    g, meta, system, ew = load("spce864")
    args = (system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    best = M.autotune(*args, g["r"][0], precision=precision)
    assert best["cells_per_cutoff"] in (1, 2, 3)
    assert best["kspace_ctas_per_sm"] in (6, 10, 16)
    ms = best["ms"]
    assert (ms[ms > 0] > 0).any()
    if best["pair_variant"] < 8:
        # the cell kernel's grid: the fastest of the grid x split trials
        assert ms[best["cells_per_cutoff"] - 1,
                  [6, 10, 16].index(best["kspace_ctas_per_sm"])] == ms[ms > 0].min()
    else:
        # the group kernel or its half-shell form: its fastest subdivision
        mg = {8: best["ms_group"], 9: best["ms_half"], 10: best["ms_half_t"]}[best["pair_variant"]]
        assert mg[best["cells_per_cutoff"] - 1] == mg[mg > 0].min()
    if precision == "fp64":
        assert (best["ms_half"] < 0).all() and (best["ms_half_t"] < 0).all()
    if precision == "mixed":
        # the Ewald chain beside or after the r-space chain, chosen with the variant
        assert best["kspace_serial"] in (0, 1)
        s = best["ms_serial"]
        assert s[best["kspace_serial"]] == s[s > 0].min()
    f0, _ = M.ForcePath(*args, precision=precision).forces(g["r"][0])
    assert best["pair_variant"] in range(11)
    f1, _ = M.ForcePath(*args, precision=precision, cells_per_cutoff=best["cells_per_cutoff"],
                        kspace_ctas_per_sm=best["kspace_ctas_per_sm"],
                        pair_variant=best["pair_variant"]).forces(g["r"][0])
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert np.sqrt(((f1 - f0) ** 2).sum() / (f0 ** 2).sum()) < tol


@pytest.mark.parametrize("variant", [1, 2, 3, 4, 5, 6, 7])
def test_pair_variants_give_the_same_forces(variant):
    """8 or 16 warps per home cell and the shared-memory spline change only
    the work split and where the table is read from"""
    g, meta, system, ew = load("spce864")
    args = (system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    f0, e0 = M.ForcePath(*args).forces(g["r"][0], measure=True)
    f1, e1 = M.ForcePath(*args, pair_variant=variant).forces(g["r"][0], measure=True)
    assert np.sqrt(((f1 - f0) ** 2).sum() / (f0 ** 2).sum()) < 1e-6
    assert abs(e1["lj"] - e0["lj"]) < 1e-6 * abs(e0["lj"])
