"""The CPU oracle against golden dumps of the reference cook binary.

Fixtures: tests/golden/*.npz, written by tests/golden/make_golden.py from
``cook -v128`` dumps (sim/simils.c:2259 dumpall; forces of every forces()
call, cook/forces.c:222).  The oracle restates cook/ljqqnp.c, sim/setss.c,
sim/erfc.c + sim/splines.c, sim/erexact.c, sim/ewald.c + ewpass*.c and
sim/constrd.c (SHAKE).
"""
import numpy as np
import pytest

from golden_cases import CASES, DIPOLE_CASES, load
from oracle import oracle as O


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


@pytest.mark.parametrize("case", CASES)
def test_forces_match_reference_dumps(case):
    g, meta, system, ew = load(case)
    assert np.allclose(system.q, g["q"], rtol=1e-11, atol=1e-9)
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    assert len(orc.kv) == meta["QN"]          # same k-vector set (Q->N)
    for d in range(g["r"].shape[0]):
        f, en = orc.forces(g["r"][d], nthreads=4)
        # dumps print 12 decimals of r and 9 of f: 1e-10 relative is the floor
        assert rel_rms(f, g["f"][d]) < 1e-10
    # En.pot of the last step (cook prints 9 significant digits)
    assert abs((en["el"] + en["lj"]) / meta["Epot_last"] - 1) < 5e-9


@pytest.mark.parametrize("case", DIPOLE_CASES)
def test_dipole_term_matches_reference_dumps(case):
    """Ewald(2)'s dipole term (sim/ewald.c:865-887): surroundings of
    dielectric constant 1, the Yeh-Berkowitz slab term along z (el.corr=4)
    and its energy-only form (el.corr=12, no force)"""
    g, meta, system, ew = load(case)
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"], epsinf=ew["epsinf"],
                   elcorr=ew["elcorr"])
    for d in range(g["r"].shape[0]):
        f, en = orc.forces(g["r"][d], nthreads=4)
        assert rel_rms(f, g["f"][d]) < 1e-10
    assert en["edip"] > 1.0          # a real term, not the tin-foil 1e-31 K
    assert abs((en["el"] + en["lj"]) / meta["Epot_last"] - 1) < 5e-9


def test_threads_agree():
    g, meta, system, ew = load("spce216")
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    f1, e1 = orc.forces(g["r"][0], nthreads=1)
    f4, e4 = orc.forces(g["r"][0], nthreads=4)
    assert rel_rms(f4, f1) < 1e-13
    assert abs(e4["el"] - e1["el"]) < 1e-9 * abs(e1["el"])


def test_shake_step_matches_reference_trajectory():
    g, meta, system, ew = load("spce216")
    p = meta["params"]
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    R, F = g["r"], g["f"]
    # dumps 1,2,3 are r(t0), r(t0+h), r(t0+2h) (dump 0 is the initial rhs call)
    r1 = R[2] - R[1]
    rn, r1n, it, ek = orc.shake_step(R[2], r1, F[2], p["h"], eps=p["epsc"],
                                     omega=meta["omegac"] / 2)
    assert it > 0
    assert np.abs(rn - R[3]).max() < 1e-9


def test_leapfrog_kinetic_energy_matches_reference():
    """VERLET=3 kinetic energy m (V1^2+V2^2)/(4 h^2) of sim/shakev3.c; cook
    prints En.kin of the last step (9 significant digits)"""
    g, meta, system, ew = load("spce216")
    p = meta["params"]
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    R, F = g["r"], g["f"]
    _, _, it, ek = orc.shake_step(R[3], R[3] - R[2], F[3], p["h"], eps=p["epsc"],
                                  omega=meta["omegac"] / 2)
    assert abs(ek / meta["Ekin_last"] - 1) < 5e-9


def test_virial_is_volume_derivative():
    """trace(Pvir) = -dE/dln(s) for an affine scaling r->s r, L->s L with the
    Ewald parameters and the integer k-vector set fixed.  Central finite
    differences on the total energy pin the Pvir bookkeeping restated from
    cook/ljqqnp.c MADDFORCES and sim/ewald.c:852-856.  Only the energy spline
    is shifted (rshift=1): the energy is then continuous at the cutoff and the
    force is its exact derivative."""
    g, meta, system, ew = load("spce216")
    r = g["r"][1]
    cut, alpha, kap = ew["cutoff"], ew["alpha"], ew["kappa"]
    orc = O.Oracle(system, ew["L"], cut, alpha, kap, rshift=1)
    _, en = orc.forces(r)
    W = sum(en["Pvir"][:3])
    h = 1e-5
    E = []
    for s in (1 + h, 1 - h):
        o = O.Oracle(system, ew["L"] * s, cut, alpha, kap / s, rshift=1)
        assert len(o.kv) == len(orc.kv)
        _, e = o.forces(r * s)
        E.append(e["el"] + e["lj"])
    Wfd = -(E[0] - E[1]) / (2 * h)
    # spline (erd vs d eru/dr) consistency is ~1e-7 of the large r-space terms
    assert abs(Wfd - W) < 1e-5 * abs(W)


def test_erfc_spline_against_libm():
    import math
    L = O.lib()
    import ctypes as C
    alpha, grid, cutoff, rplus = 0.26, 256, 12.0, 2.5
    n = L.orc_erfc_ntab(grid, cutoff + rplus, alpha)
    tab = np.zeros(6 * n)
    sg = C.c_double()
    L.orc_erfc_build(grid, cutoff + rplus, cutoff, alpha, 0, O._dp(tab), C.byref(sg))
    # the hyperbolic spline on grid 256 (in alpha^2 r^2) is good to ~1e-7
    # relative from 2 A on (the shortest intermolecular distances)
    for r in np.linspace(2.0, cutoff, 97):
        rr = r * r
        exact = math.erfc(alpha * r) / r
        assert abs(L.orc_eru(O._dp(tab), sg.value, rr) - exact) < 1e-7 * exact


def test_drude_forces_match_reference_dumps():
    """POLAR build of cook (cook/ljqqpol.c pair terms, Drude charges in the
    Ewald sums): centre and Drude forces at cook's predicted shell positions"""
    g, meta, system, ew = load("drude216")
    assert np.allclose(system.qpol, g["qD"], rtol=1e-11, atol=1e-9)
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    for d in range(g["r"].shape[0]):
        r2 = np.vstack([g["r"][d], g["rD"][d]])
        f2, _ = orc.forces(r2, nthreads=4)
        fr = np.vstack([g["f"][d], g["fD"][d]])
        assert rel_rms(f2, fr) < 1e-10


def test_aspc_scf_chain_matches_reference():
    """ASPC k=2 predictor (sim/pred2.c) over SCF-corrected shell positions
    (sim/scf.c selffield, omega=4/7) reproduces cook's predicted positions"""
    g, meta, system, ew = load("drude216")
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    ns = system.ns
    B, om = O.aspc_coef(2)
    assert np.allclose(B, [2.8, -2.8, 1.2, -0.2]) and abs(om - 4 / 7) < 1e-15
    corr = {}
    for t in range(1, g["r"].shape[0]):
        r2 = np.vstack([g["r"][t], g["rD"][t]])
        f2 = np.vstack([g["f"][t], g["fD"][t]])
        r2c, _, _, _ = orc.selffield(r2, f2, om if t > 1 else 0.6)
        corr[t] = r2c[ns:]
    for t in range(5, g["r"].shape[0]):
        pred = sum(B[i] * corr[t - 1 - i] for i in range(4))
        assert np.abs(pred - g["rD"][t]).max() < 1e-10


def test_dependant_positions_in_reference_dumps():
    """cook dumps r after depend_r: every TIP4P/2005 charge site M sits at
    (1-2w) O + w H1 + w H2 (sim/norm.c:1188-1193)"""
    g, meta, system, ew = load("tip4p216")
    assert system.ndep == 216
    for d in range(g["r"].shape[0]):
        assert np.abs(O.depend_r(system, g["r"][d]) - g["r"][d]).max() < 1e-10


def test_dependant_step_matches_reference_trajectory():
    """leap-frog + SHAKE of TIP4P/2005 with the M-site force moved onto O, H,
    H before the step (sim/constrd.c:747) and M placed after it"""
    g, meta, system, ew = load("tip4p216")
    p = meta["params"]
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    R, F = g["r"], g["f"]
    f = O.depend_f(system, F[2])
    # the redistribution keeps the total force and the torque about any point
    dep = system.dep_site
    assert np.allclose(f.sum(0) - f[dep].sum(0), F[2].sum(0), atol=1e-7)
    rn, r1n, it, ek = orc.shake_step(R[2], R[2] - R[1], f, p["h"], eps=p["epsc"],
                                     omega=meta["omegac"] / 2)
    rn = O.depend_r(system, rn)
    assert it > 0
    assert np.abs(rn - R[3]).max() < 1e-9
    # VERLET=3 kinetic energy of the last step (massless M contributes none)
    _, _, _, ek = orc.shake_step(R[3], R[3] - R[2], O.depend_f(system, F[3]), p["h"],
                                 eps=p["epsc"], omega=meta["omegac"] / 2)
    assert abs(ek / meta["Ekin_last"] - 1) < 5e-9


def test_out_of_plane_dependants_match_reference():
    """the test model T5R (two "Lone" and one "Rowlinson" dependant per
    rigid water, sim/norm.c:1196-1231, 1304-1360): cook's dumped positions
    of the dependants follow from their parents; its step from the forces
    moved onto O, H, H keeps the total force and gives cook's next
    positions"""
    g, meta, system, ew = load("t5r216")
    assert system.ndep == 648 and set(system.dep_type.tolist()) == {1, 2}
    for d in range(g["r"].shape[0]):
        assert np.abs(O.depend_r(system, g["r"][d]) - g["r"][d]).max() < 1e-10
    p = meta["params"]
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    R, F = g["r"], g["f"]
    f = O.depend_f(system, F[2], R[2])
    dep = system.dep_site
    assert np.allclose(f.sum(0) - f[dep].sum(0), F[2].sum(0), atol=1e-7)
    rn, _, it, _ = orc.shake_step(R[2], R[2] - R[1], f, p["h"], eps=p["epsc"],
                                  omega=meta["omegac"] / 2)
    rn = O.depend_r(system, O.normalize(system, rn, ew["L"]))
    assert it > 0
    assert np.abs(rn - R[3]).max() < 1e-9


def test_reference_states_are_normalized():
    """cook's dumped positions are normalized: every molecule's lowest
    massive-site coordinate lies in [r0, r0 + L) with r0 = 0.15 (the value
    cook picks for Verlet/SHAKE), so the oracle's normalize leaves them alone"""
    for case in ("spce216", "brine532", "tip4p216"):
        g, meta, system, ew = load(case)
        for d in range(g["r"].shape[0]):
            assert np.array_equal(O.normalize(system, g["r"][d], ew["L"]), g["r"][d])


def test_nose_hoover_trajectory_matches_reference():
    """cook's Nose-Hoover Verlet+SHAKE (thermostat=2, tau.T 0.05 ps, TRVP
    k -> 2): five steps from r(t0) and the initial r1 of cook's velocity
    playback (float32) reproduce cook's positions; cook's printed En.kin of
    the last step (the thermostat changes it from the NVE value)"""
    g, meta, system, ew = load("nose216")
    p = meta["params"]
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    h = p["h"]
    nh = O.NoseHoover(298.0, 0.05, 3 * system.ns - len(system.cons) - 3, h)
    r = g["r"][1].copy()
    r1 = g["vlb_r"][0].astype(np.float64) * h
    for step in range(5):
        f, _ = orc.forces(r, measure=False, nthreads=4)
        r, r1, it, ek = nh.step(orc, r, r1, f, omega=meta["omegac"] / 2)
        ref = g["r"][step + 2] if step + 2 < g["r"].shape[0] else g["plb_r"][5]
        # dumps print 12 decimals, the playback frame is float32
        tol = 5e-8 if step + 2 < g["r"].shape[0] else 3e-6
        assert np.abs(r - ref).max() < tol, step
    assert nh.k == 2 and nh.logsv != 0
    # the last step's kinetic energy (9 digits printed); the initial r1 is
    # known to float precision only
    assert abs(ek / meta["Ekin_last"] - 1) < 1e-8


def test_bounddr_and_drift_removal_match_reference_trajectory():
    """cook with drmax = -0.02 A: after every step bounddr scales the step of
    every faster site down to 0.02 A (sim/norm.c:1513-1560), then the
    momentum drift that this creates is removed (removedrifts, momentum bits,
    once per cycle = every step here, sim/maincps.c:65)"""
    g, meta, system, ew = load("bounddr216")
    p = meta["params"]
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    R = g["r"]
    r1, n, q = O.bounddr(R[2] - R[1], p["drmax"])
    assert n > 100 and q < 0.5
    r1, _ = O.remove_drift(system, r1)
    r = R[2]
    for k in range(2):
        f, _ = orc.forces(r, measure=False, nthreads=4)
        r, r1, it, ek = orc.shake_step(r, r1, f, p["h"], eps=p["epsc"], omega=meta["omegac"] / 2)
        assert np.abs(r - R[3 + k]).max() < 1e-9
        r1, n, q = O.bounddr(r1, p["drmax"])
        r1, _ = O.remove_drift(system, r1)
