"""Seeded synthetic starting configurations (cook ``init="crystal"`` analogue).

Molecule anchors (the first site, O for water) sit on an fcc lattice filling
the box; each molecule gets a uniformly random orientation and rigid-body
Maxwell velocities (centre-of-mass translation + rotation) at temperature T.
Ions replace randomly chosen lattice molecules.  Returns cook's state pair
r = r(t), r1 = r(t) - r(t-h) = h v, in the site order of ``forcefield``.
"""
import math

import numpy as np

from . import forcefield as ff

AVOGADRO = 6.02214076e23


def box_length(species, counts, density):
    """cubic box edge (A) of the given composition at density (g/cm^3)"""
    m = 0.0
    for s, n in zip(species, counts):
        sp = ff.SPECIES[s]()
        m += n * sum(ff.ble_type_row(t)[0] for t in sp.sites)
    V = m / (density * AVOGADRO * 1e-24)
    return V ** (1.0 / 3.0)


def _random_rotations(rng, n):
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1)[:, None]
    w, x, y, z = q.T
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def build(species, counts, L, seed=0, T=298.0, h=0.002):
    """system, r [ns,3], r1 [ns,3] for the species/counts in a cubic box L"""
    rng = np.random.default_rng(seed)
    system = ff.build_system(species, counts)
    nmol = sum(counts)
    n = 1
    while 4 * n ** 3 < nmol:
        n += 1
    a = L / n
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    cells = np.array([[i, j, k] for i in range(n) for j in range(n) for k in range(n)], float)
    sites = ((cells[:, None, :] + base[None, :, :]).reshape(-1, 3) + 0.25) * a
    pick = rng.permutation(len(sites))[:nmol]
    anchors = sites[pick]
    r = np.zeros((system.ns, 3))
    r1 = np.zeros((system.ns, 3))
    imol = 0
    for s, cnt in zip(species, counts):
        sp = ff.SPECIES[s]()
        geo = sp.geometry - sp.geometry[0]
        m = np.array([ff.ble_type_row(t)[0] / ff.MUNIT for t in sp.sites])
        Rm = _random_rotations(rng, cnt)
        for k in range(cnt):
            i0 = system.mol_first[imol]
            x = anchors[imol] + geo @ Rm[k].T
            com = (m[:, None] * x).sum(0) / m.sum()
            v = rng.normal(size=3) * math.sqrt(T / m.sum())
            if len(m) > 1:
                d = x - com
                I = (m[:, None] * d * d).sum() * 2.0 / 3.0
                omega = rng.normal(size=3) * math.sqrt(T / I)
                v = v + np.cross(omega, d)
            r[i0:i0 + len(m)] = x
            r1[i0:i0 + len(m)] = h * v
            imol += 1
    # remove the total momentum (cook: "Remove v drifts")
    p = (system.mass[:, None] * r1).sum(0) / system.mass.sum()
    r1 -= p
    return system, r, r1


WORKLOADS = {
    # the 864 SPC/E configuration (L = 29.65 A, cutoff 12, alpha 0.26, |n|<=8)
    "spce864": dict(species=["WAT"], counts=[864], L=29.65, cutoff=12.0, alpha=0.26, kn=8),
    # brine: 4096 SPC/E + 128 Na+ + 128 Cl- at 1.06 g/cm3, cutoff 10, alpha 0.31, |n|<=12
    "brine4352": dict(species=["WAT", "NA", "CL"], counts=[4096, 128, 128], density=1.06,
                      cutoff=10.0, alpha=0.31, kn=12),
    # 32768 SPC/E waters at 0.997 g/cm3 (L = 99.44 A), cutoff 12, alpha 0.26, |n|<=20
    "spce32768": dict(species=["WAT"], counts=[32768], density=0.997, cutoff=12.0, alpha=0.26,
                      kn=20),
    # the same box of Drude-polarizable waters (shell on O, q_D -1.8 e,
    # k 4184 kJ/mol/A^2, alpha 1.0759 A^3); ASPC k=2 with one SCF iteration
    # per step
    "drude32768": dict(species=["WATD"], counts=[32768], density=0.997, cutoff=12.0,
                       alpha=0.26, kn=20, aspc_k=2, scf_iter=1),
}


def workload(name, seed=0, T=298.0, h=0.002):
    """a named workload; for Drude systems r and r1 carry the shell
    displacements (zero: shells start on their sites) after the sites"""
    w = WORKLOADS[name]
    L = w.get("L") or box_length(w["species"], w["counts"], w["density"])
    system, r, r1 = build(w["species"], w["counts"], L, seed=seed, T=T, h=h)
    if system.polar:
        r = np.vstack([r, np.zeros_like(r)])
        r1 = np.vstack([r1, np.zeros_like(r1)])
    return dict(name=name, system=system, r=r, r1=r1, L=L, cutoff=w["cutoff"], alpha=w["alpha"],
                kappa=(w["kn"] + 1e-6) / L, h=h, kn=w["kn"], aspc_k=w.get("aspc_k", 2),
                scf_iter=w.get("scf_iter", 1))


def equilibrate(w, steps=400, T=298.0, every=20, h=None, polar_steps=200, **kw):
    """Relax a lattice start with rigid (non-polarizable) molecules on the
    GPU: leap-frog + SHAKE with the half-step velocities rescaled to T every
    ``every`` steps.  Drude systems are relaxed as their SPC/E parents and
    get their shells back on the sites.  Returns the workload with new r, r1."""
    import macsimus_gb300 as M
    system = w["system"]
    ns = system.ns
    rigid = system
    if system.polar:
        rigid = ff.build_system([s.replace("WATD", "WAT") for s in system.species],
                                system.counts)
    hh = h or w["h"]
    fp = M.ForcePath(rigid, [w["L"]] * 3, w["cutoff"], w["alpha"], w["kappa"],
                     precision="mixed", h=hh, epsc=1e-7, **kw)
    r, r1 = w["r"][:ns].copy(), w["r1"][:ns].copy() * (hh / w["h"])
    nf = 6 * rigid.nmol - 3 if len(rigid.cons_len) else 3 * ns - 3
    m = rigid.mass[:, None]
    for _ in range(steps // every):
        fp.md_set_state(r, r1)
        fp.md_steps(every, measure=False)
        r, r1 = fp.md_get_state()
        ekin = 0.5 * (m * (r1 / hh) ** 2).sum()
        Tnow = 2 * ekin / nf
        r1 *= np.sqrt(T / max(Tnow, 1e-6))
    fp.close()
    out = dict(w)
    if system.polar:
        # then the polarizable system itself, still with velocity rescaling,
        # to absorb the polarization energy released when shells switch on
        r = np.vstack([r, np.zeros_like(r)])
        r1 = np.vstack([r1, np.zeros_like(r1)])
        fpp = M.ForcePath(system, [w["L"]] * 3, w["cutoff"], w["alpha"], w["kappa"],
                          precision="mixed", h=hh, epsc=1e-7, aspc_k=w.get("aspc_k", 2),
                          scf_iter=w.get("scf_iter", 1), **kw)
        for _ in range(polar_steps // every):
            fpp.md_set_state(r, r1)
            fpp.md_steps(every, measure=False)
            r, r1 = fpp.md_get_state()
            ekin = 0.5 * (m * (r1[:ns] / hh) ** 2).sum()
            Tnow = 2 * ekin / nf
            r1[:ns] *= np.sqrt(T / max(Tnow, 1e-6))
        fpp.close()
    r1[:ns] *= w["h"] / hh
    out["r"], out["r1"] = r, r1
    out["equilibrated"] = steps + (polar_steps if system.polar else 0)
    return out


def ionic_boxes(nbox=256, seed=0, T=298.0, h=0.002, nmin=500, nmax=4000, rho_star=0.8):
    """Independent LJ + point-charge ionic-fluid boxes: per box N uniform in
    [nmin, nmax] (even, equimolar +-1 e), sigma uniform in [3.0, 4.5] A and
    epsilon in [0.1, 1.0] kJ/mol for each ion type, number density
    rho_star / sigma_mean^3, cutoff 2.5 sigma_max (at most 0.49 L), Ewald
    alpha = 3.1/cutoff and |n| <= 1.08 alpha L (erfc and Gaussian tails
    ~1e-5 at the cutoffs).  Ions start on a simple cubic lattice, randomly
    assigned, with Maxwell velocities at T (zero total momentum)."""
    rng = np.random.default_rng(seed)
    out = []
    for b in range(nbox):
        n = 2 * int(rng.integers(nmin // 2, nmax // 2 + 1))
        sp, sm = rng.uniform(3.0, 4.5, 2)
        ep, em = rng.uniform(0.1, 1.0, 2)
        system = ff.ionic_system(n, sp, ep, sm, em)
        smean = 0.5 * (sp + sm)
        L = (n * smean ** 3 / rho_star) ** (1.0 / 3.0)
        cutoff = min(2.5 * max(sp, sm), 0.49 * L)
        alpha = 3.1 / cutoff
        kn = int(math.ceil(1.08 * alpha * L))
        m = 1
        while m ** 3 < n:
            m += 1
        grid = (np.array([[i, j, k] for i in range(m) for j in range(m) for k in range(m)], float)
                + 0.5) * (L / m)
        pick = rng.permutation(len(grid))[:n]
        r = grid[pick][rng.permutation(n)]
        v = rng.normal(size=(n, 3)) * np.sqrt(T / system.mass)[:, None]
        v -= (system.mass[:, None] * v).sum(0) / system.mass.sum()
        out.append(dict(name="ionic%d" % b, system=system, r=r, r1=h * v, L=L, cutoff=cutoff,
                        alpha=alpha, kappa=(kn + 1e-6) / L, kn=kn, h=h, sigma=(sp, sm),
                        epsilon=(ep, em)))
    return out
