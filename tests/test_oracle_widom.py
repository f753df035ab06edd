"""The oracle's Widom insertion (cook/widom.c Einsert, sim/simmeas.c Widom,
sim/siminit.c Widomcutcorr) against the reference binary's output on the
same configuration (tests/golden/widom500: 1e7 insertions by cook).

The reference draws its insertion points from its own generator, so the
Widom average is compared statistically (both estimate the same quantity on
the same configuration); the cutoff correction is compared exactly."""
import numpy as np

from golden_cases import load
from macsimus_gb300 import forcefield as ff
from oracle import oracle as O


def setup():
    g, meta, system, ew = load("widom500")
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    return g, meta, system, ew, orc


PRB = [ff.TYPE_ORDER.index("PRB")]


def test_cutoff_correction_matches_cook():
    g, meta, system, ew, orc = setup()
    _, corr, _ = orc.widom(g["r"][-1], PRB, [0.0], [0, 0, 0], 10, 1, 298.0)
    # cook prints corr with %g (6 significant digits)
    assert abs(corr - meta["widom"]["corr"]) <= 5e-6 * abs(meta["widom"]["corr"])


def test_widom_average_matches_cook_statistically():
    g, meta, system, ew, orc = setup()
    n, T = 2_000_000, 298.0
    s, corr, U = orc.widom(g["r"][-1], PRB, [0.0], [0, 0, 0], n, 20231, T, energies=True)
    w = np.where(-U / T > -700, np.exp(-U / T), 0.0)
    assert abs(w.sum() - s) <= 1e-9 * s
    raw = s / n
    # relative standard errors of both estimates of <exp(-U/T)>
    sig = w.std() / raw
    err = np.sqrt(sig ** 2 / n + sig ** 2 / meta["widom"]["n"])
    raw_cook = np.exp(-meta["widom"]["mu_raw_K"] / T)
    assert abs(np.log(raw / raw_cook)) < 4 * err + 1e-5
    V = float(np.prod(ew["L"]))
    mu_kT = -np.log(raw * np.exp(-corr / (V * T)))
    assert abs(mu_kT - meta["widom"]["mu_kT"]) < 4 * err + 1e-5


def test_insertion_stream_and_energies():
    g, meta, system, ew, orc = setup()
    # one-site ghost: the point is the upper 32 bits of words 0..2 times L
    p = orc.widom_sites(99, 7, [[0, 0, 0]])[0]
    for c in range(3):
        w = O.lib().orc_widom_word(99, 7, c)
        assert p[c] == (w >> 32) / 2 ** 32 * ew["L"][c]
    # several sites: a rigid rotation of the geometry about the point
    geo = np.array([[0, 0, 0], [1.0, 0, 0], [0, 1.5, 0.5]])
    s = orc.widom_sites(99, 7, geo)
    assert np.allclose(s[0], p)
    d = s - s[0]
    assert np.allclose(np.linalg.norm(d, axis=1), np.linalg.norm(geo, axis=1), atol=1e-12)
    assert abs(np.dot(d[1], d[2]) - np.dot(geo[1], geo[2])) < 1e-12
    # the energies Widom sums are Einsert at those points
    _, _, U = orc.widom(g["r"][-1], PRB, [0.0], [0, 0, 0], 50, 5, 298.0, energies=True)
    for k in (0, 17, 49):
        pos = orc.widom_sites(5, k, [[0, 0, 0]])
        assert U[k] == orc.einsert(g["r"][-1], PRB, [0.0], pos)


def test_einsert_is_a_pair_sum():
    """Einsert of a ghost placed on top of nothing but one box site at
    distance r equals the LJ (smooth cutoff) + q q eru pair energy"""
    g, meta, system, ew, orc = setup()
    r = g["r"][-1]
    # a charged ghost of the cation type next to site 0 and far from others:
    # compare with the energy difference of the full sums at two points
    pos = r[0] + np.array([3.1, 0.0, 0.0])
    e_full = orc.einsert(r, [ff.TYPE_ORDER.index("AP")], [0.0], pos[None])
    # removing site 0 from the box changes Einsert by its pair term
    keep = np.arange(1, system.ns)
    sys2 = ff.build_system(["AP", "AM", "PRB"], [249, 250, 0])
    orc2 = O.Oracle(sys2, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    e_rest = orc2.einsert(r[keep], [ff.TYPE_ORDER.index("AP")], [0.0], pos[None])
    ss = orc.ss[ff.TYPE_ORDER.index("AP") * len(system.typeE) + system.type[0]]
    rr = 3.1 ** 2
    x = ss.Sq / rr
    y = x ** 3
    u = ss.E4 * (y * y - y) if rr < ss.C1q else ss.A * (rr - ss.C2q) ** 2
    assert abs((e_full - e_rest) - u) < 1e-9 * abs(u)


def test_identity_change_matches_cook():
    """cook's XWidom (sim/simmeas.c:1961, cook/widom.c Eidchange): every AP
    cation of the last configuration turned into APV (sigma 3.3 -> 3.4 A,
    epsilon 0.5 -> 0.55 kJ/mol, charge +1 -> +0.8 e); cook prints
    mu = -T ln <exp(-dU/T)> to 6 significant digits"""
    g, meta, system, ew = load("xwidom500")
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    T = 298.0
    ap = list(range(system.counts[0]))   # molecules run species by species
    assert system.species[0] == "AP" and len(ap) == 250
    vt = [ff.TYPE_ORDER.index("APV")]
    vq = [0.8 * ff.ELECTRON]
    s, dU = orc.xwidom(g["r"][-1], ap, vt, vq, T)
    mu = -T * np.log(s / len(ap))
    assert abs(mu - meta["xwidom"]["mu_raw_K"]) <= 6e-6 * abs(meta["xwidom"]["mu_raw_K"])
    assert np.isclose(s, np.exp(-dU / T).sum(), rtol=1e-12)
