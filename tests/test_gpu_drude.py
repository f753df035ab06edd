"""Drude (shell) polarizable water on the GPU against the oracle and cook's
POLAR dumps: the four-term polar pair kernel and the Drude charges in the
Ewald sums (cook/ljqqpol.c, sim/ewald.c), the SCF iteration (sim/scf.c
selffield) and the ASPC + SCF + SHAKE step (sim/pred2.c, sim/constrd.c)."""
import numpy as np
import pytest

import macsimus_gb300 as M
from golden_cases import load
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-5


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


def setup(precision, **kw):
    g, meta, system, ew = load("drude216")
    fp = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"],
                     precision=precision, h=meta["params"]["h"], epsc=meta["params"]["epsc"],
                     omegac=meta["omegac"], **kw)
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    return g, meta, system, ew, fp, orc


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_drude_forces(precision):
    g, meta, system, ew, fp, orc = setup(precision)
    tol = 1e-10 if precision == "fp64" else MIXED_TOL
    for d in (1, g["r"].shape[0] - 1):
        r2 = np.vstack([g["r"][d], g["rD"][d]])
        f2, en = fp.forces(r2, measure=True)
        fo, eo = orc.forces(r2, nthreads=4)
        fr = np.vstack([g["f"][d], g["fD"][d]])
        assert rel_rms(f2, fo) < tol
        assert rel_rms(f2, fr) < max(tol, 2e-10)
        etol = 1e-10 if precision == "fp64" else 2e-6
        for k in ("el", "er", "ek"):
            assert abs(en[k] - eo[k]) <= etol * abs(eo["eself"]), k
        assert abs(en["lj"] - eo["lj"]) <= (1e-10 if precision == "fp64" else 1e-5) * abs(eo["lj"])


@pytest.mark.parametrize("variant", [8, 9, 10])
def test_drude_group_kernels(variant):
    """the group kernel (8) and its half-shell form (9: every pair once, the
    neighbour's centre and shell forces in fixed point) with Drude shells:
    the oracle's centre and shell forces, energies and virial, as the cell
    kernel gives them; bit-reproducible"""
    g, meta, system, ew, fp, orc = setup("mixed", pair_variant=variant)
    for d in (1, g["r"].shape[0] - 1):
        r2 = np.vstack([g["r"][d], g["rD"][d]])
        f2, en = fp.forces(r2, measure=True)
        fo, eo = orc.forces(r2, nthreads=4)
        ns = system.ns
        assert rel_rms(f2, fo) < MIXED_TOL
        assert rel_rms(f2[ns:], fo[ns:]) < MIXED_TOL   # the shells alone
        for k in ("el", "er", "ek"):
            assert abs(en[k] - eo[k]) <= 2e-6 * abs(eo["eself"]), k
        assert abs(en["lj"] - eo["lj"]) <= 1e-5 * abs(eo["lj"])
        for m in range(6):
            assert abs(en["Pvir"][m] - eo["Pvir"][m]) <= 2e-5 * abs(eo["Pvir"][0]), m
        f3, _ = fp.forces(r2, measure=True)
        assert np.array_equal(f3, f2)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_selffield_iteration(precision):
    g, meta, system, ew, fp, orc = setup(precision)
    r2 = np.vstack([g["r"][3], g["rD"][3]])
    f2, en = fp.forces(r2, measure=True)
    fo, eo = orc.forces(r2)
    om = 4.0 / 7.0
    rg, fg, eg = fp.selffield(r2, f2, om, en)
    ro, fo2, eo2, _ = orc.selffield(r2.copy(), fo.copy(), om, eo)
    ns = system.ns
    tol = 1e-10 if precision == "fp64" else MIXED_TOL
    # new shell positions (displacements are ~0.1 A) and folded forces
    assert np.abs(rg[ns:] - ro[ns:]).max() < (1e-12 if precision == "fp64" else 1e-7)
    assert rel_rms(fg[:ns], fo2[:ns]) < tol
    assert abs(eg["self"] - eo2["self"]) < (1e-9 if precision == "fp64" else 1e-5) * abs(eo2["self"])
    assert abs(eg["el"] - eo2["el"]) < (1e-10 if precision == "fp64" else 2e-6) * abs(eo["eself"])


def oracle_md(orc, system, r, r1, h, k, niter, nsteps, epsc, omegac):
    """ASPC + SCF + SHAKE with the oracle, the sequence of sim/constrd.c"""
    ns = system.ns
    hist = [np.zeros((ns, 3)) for _ in range(k + 2)]
    hist[0] = r[ns:].copy()
    hist[k + 1] = r1[ns:].copy()
    hp, kk = 0, 0
    om = 0.6
    r, r1 = r.copy(), r1.copy()
    K2 = k + 2
    for _ in range(nsteps):
        B, _ = O.aspc_coef(kk)
        pred = sum(B[i] * hist[(hp - i) % K2] for i in range(kk + 2))
        if kk < k:
            kk += 1
            om = O.aspc_coef(kk)[1]
        r2 = np.vstack([r[:ns], pred])
        for _ in range(niter):
            f2, _ = orc.forces(r2, measure=False, nthreads=4)
            r2, f2, _, _ = orc.selffield(r2, f2, om)
        hp = (hp + 1) % K2
        hist[hp] = r2[ns:].copy()
        rs, r1s, it, ek = orc.shake_step(r2[:ns], r1[:ns], f2[:ns], h, eps=epsc,
                                         omega=omegac / 2)
        r = np.vstack([rs, r2[ns:]])
        r1 = np.vstack([r1s, r1[ns:]])
    return r


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_aspc_md_matches_oracle(precision):
    g, meta, system, ew, fp, orc = setup(precision, aspc_k=2, scf_iter=1)
    ns = system.ns
    R, RD = g["r"], g["rD"]
    r = np.vstack([R[4], RD[4]])
    r1 = np.vstack([R[4] - R[3], RD[3]])
    fp.md_set_state(r, r1)
    en = fp.md_steps(4)
    rg, _ = fp.md_get_state()
    ro = oracle_md(orc, system, r, r1, meta["params"]["h"], 2, 1, 4, meta["params"]["epsc"],
                   meta["omegac"])
    tol = 1e-9 if precision == "fp64" else 1e-6
    assert np.abs(rg[:ns] - ro[:ns]).max() < tol
    assert np.abs(rg[ns:] - ro[ns:]).max() < tol
    assert np.isfinite(en["self"]) and en["self"] > 0


def test_shell_escape_is_reported_not_fatal():
    """a shell pushed beyond el.minqq (1 A) is reported as MG_ERR_SCF, as
    cook stops with "DRUDE new cfg" (sim/scf.c:253); the context stays usable"""
    g, meta, system, ew, fp, orc = setup("fp64")
    ns = system.ns
    r2 = np.vstack([g["r"][3], g["rD"][3]])
    f2, en = fp.forces(r2, measure=True)
    bad = f2.copy()
    bad[ns:] *= 1e4          # a huge field on the shells
    with pytest.raises(M.MGError) as e:
        fp.selffield(r2, bad, 0.6)
    assert e.value.code == 7
    f3, _ = fp.forces(r2)
    assert rel_rms(f3, f2) < 1e-12
