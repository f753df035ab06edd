"""Force-field tables and system layout in MACSIMUS cook conventions.

Host-side counterpart of the parts of cook/simdef.c (``readblend``) that the
force path consumes: per-type Lennard-Jones parameters (EvdW<0 in K, RvdW in
Angstrom, polarizability ``alpha`` for the combining rule), site charges in
program units (e * 408.779826922048, sim/units.h:101-108), site masses in
program units (g/mol / 0.831446261815324, cook/simdef.c:1021) and the rigid
bond constraints of each species.

Numbers pass through the same decimal text a cook ``.ble`` file holds
(12 significant digits for LJ parameters, cook/simdef.c:620-628), so a system
built here and the same system read by cook from the written ``.ble`` carry
identical doubles.  ``ble_text`` writes that file.
"""
import math
from dataclasses import dataclass, field

import numpy as np

ELECTRON = 408.779826922048        # charge of e in program units
MUNIT = 0.831446261815324          # g/mol per program mass unit
EUNIT = 8.31446261815324           # J/mol per program energy unit (K)
KCAL = 4184.0
KJ_PER_KCAL = 4.184
EUNIT_KCAL = KCAL / EUNIT          # cook's default eunit: kcal/mol -> K
HOH = math.sqrt(8.0 / 3.0)         # SPC/E H-H distance (O-H 1 A, tetrahedral)


def _g12(x):
    return float("%.12g" % x)


def rvdw_of_sigma(sigma):
    """van der Waals radius of the .ble table: sigma * 2^(1/6) / 2."""
    return sigma * 2.0 ** (1.0 / 6.0) / 2.0


# LJ site types: name -> (mass g/mol, epsilon kJ/mol, sigma A)
SITE_TYPES = {
    "H": (1.008, 0.0, 0.0),
    "O": (15.9994, 0.6502, 3.166),
    "NA": (22.9898, 1.475, 2.16),
    "CL": (35.453, 0.0535, 4.83),
    "OD": (15.9994, 0.6502, 3.166),   # oxygen carrying a Drude charge
    # a model ionic fluid (LJ spheres with +-1 e) and a neutral LJ probe for
    # Widom insertions (sigma 3.2 A, epsilon 0.65 kJ/mol)
    "AP": (22.9898, 0.5, 3.3),
    "AM": (35.453, 0.7, 4.1),
    "PRB": (39.948, 0.65, 3.2),
    # the cation with changed size, well depth and charge: the target of an
    # identity change (XWidom) of AP
    "APV": (22.9898, 0.55, 3.4),
    # TIP4P/2005: the LJ oxygen and the massless charge site M
    "OT": (15.9994, 0.774908, 3.1589),
    "MW": (0.0, 0.0, 0.0),
}
TYPE_ORDER = ["H", "O", "NA", "CL", "OD", "AP", "AM", "PRB", "OT", "MW", "APV"]

# Drude parameters of a site type: (alphapol A^3, chargepol e).  The Drude
# water has the shell charge -1.8 e on a spring of 4184 kJ/mol/A^2
# (1000 kcal/mol/A^2); its polarizability follows as
# alpha = q^2/(4 pi eps0 k) = 1.8^2 * 332.06371330/1000 A^3 (sim/units.h:90).
DRUDE_QD = -1.8
DRUDE_K_KCAL = 1000.0
TYPE_DRUDE = {"OD": (DRUDE_QD ** 2 * 332.06371330 / DRUDE_K_KCAL, DRUDE_QD)}


def ble_type_row(name):
    """(mass, EvdW[kcal/mol], RvdW[A]) exactly as written into the .ble."""
    m, eps, sig = SITE_TYPES[name]
    ev = _g12(-eps / KJ_PER_KCAL)
    rv = _g12(rvdw_of_sigma(sig)) if sig else 0.5
    return float("%.6f" % m), ev, rv


def type_table():
    """Per-type arrays in program units: EvdW [K] (<=0), RvdW [A], alpha."""
    E, R, A, M = [], [], [], []
    for n in TYPE_ORDER:
        m, ev, rv = ble_type_row(n)
        E.append(EUNIT_KCAL * ev)
        R.append(rv)
        A.append(0.0)
        M.append(m)
    return np.array(E), np.array(R), np.array(A), np.array(M)


@dataclass
class Species:
    name: str
    sites: list            # type names
    charges: list          # e
    geometry: np.ndarray   # reference geometry [ns,3] (A)
    bonds: list = field(default_factory=list)  # (i, j, length)
    drude: dict = None     # {site index: (alphapol A^3, chargepol e)}
    # dependants: (site, [(parent, weight), ...]) for a linear ("Middle")
    # one; (site, [3 parents], "R", {"wz": .}) for a Rowlinson one (above
    # parent 0 along the normal of the parents' plane); (site, [3 parents],
    # "L", {"x", "y", "wz", "tx", "ty"}) for a Lone (out-of-plane) one
    # (cook/simdef.c:322-432; sim/norm.c:1161-1360)
    dependants: list = field(default_factory=list)


DEP_KINDS = {"M": 0, "R": 1, "L": 2}


def dep_parameters(kind, extra):
    """the 13 parameters of a Rowlinson or Lone dependant as cook reads them
    from the .ble (printed with 15 digits, then the coefficient vectors
    x, y, tx, ty shifted to zero sum, cook/simdef.c:313-320): wz, x[3],
    y[3], tx[3], ty[3] (zeros where unused)"""
    par = np.zeros(13)
    if kind == "M":
        return par
    par[0] = float("%.15g" % extra["wz"])
    if kind == "L":
        for o, key in ((1, "x"), (4, "y"), (7, "tx"), (10, "ty")):
            v = [float("%.15g" % c) for c in extra[key]]
            sm = (v[0] + v[1] + v[2]) / 3
            par[o:o + 3] = [v[0] - sm, v[1] - sm, v[2] - sm]
    return par


def spce():
    c = math.cos(math.acos(-1.0 / 3.0))
    s = math.sin(math.acos(-1.0 / 3.0))
    return Species("WAT", ["O", "H", "H"], [-0.8476, 0.4238, 0.4238],
                   np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [c, s, 0.0]]),
                   bonds=[(0, 1, 1.0), (0, 2, 1.0), (1, 2, HOH)])


def tip4p2005():
    """TIP4P/2005 water: O (LJ), H, H, and the massless charge site M on the
    bisector, 0.1546 A from O, a linear dependant of O, H, H"""
    a = math.radians(104.52)
    doh = 0.9572
    h1 = np.array([doh, 0.0, 0.0])
    h2 = np.array([doh * math.cos(a), doh * math.sin(a), 0.0])
    bis = 0.5 * (h1 + h2)
    w = 0.1546 / (2 * np.linalg.norm(bis))
    m = w * (h1 + h2)
    dhh = float(np.linalg.norm(h1 - h2))
    sp = Species("T4P", ["OT", "H", "H", "MW"], [0.0, 0.5564, 0.5564, -1.1128],
                 np.array([[0.0, 0.0, 0.0], h1, h2, m]),
                 bonds=[(0, 1, doh), (0, 2, doh), (1, 2, dhh)])
    sp.dependants = [(3, [(0, 1 - 2 * w), (1, w), (2, w)])]
    return sp


def water_lone_rowlinson():
    """A test model for the out-of-plane dependants (no reference example
    uses them): the rigid TIP4P/2005 geometry with O (LJ), H, H, two "Lone"
    sites 0.3 A behind O along the bisector and 0.5 A above and below the
    molecular plane, and a "Rowlinson" site 0.25 A above O along the
    normal, charged so that the molecule is neutral.  The Lone frame is
    xx = H1 - H2, yy = (H1 + H2)/2 - O (orthogonal for the symmetric
    molecule); tx, ty make the normal forces on O, H, H reproduce the torque
    of the dependant's force about its in-plane point: sum tx = sum ty = 0,
    sum tx a = sum ty b = -wz, sum tx b = sum ty a = 0 with (a, b) the
    parents' coordinates in that frame (the conditions of sim/norm.c:1338-1360
    for a rigid triangle)"""
    a = math.radians(104.52)
    doh = 0.9572
    o = np.zeros(3)
    h1 = np.array([doh, 0.0, 0.0])
    h2 = np.array([doh * math.cos(a), doh * math.sin(a), 0.0])
    bis = 0.5 * (h1 + h2) - o
    sb = -0.3 / float(np.linalg.norm(bis))
    w = [1 - sb, 0.5 * sb, 0.5 * sb]
    x, y = [0.0, 1.0, -1.0], [-1.0, 0.5, 0.5]
    xx = h1 - h2
    yy = bis
    zhat = np.cross(xx, yy) / np.linalg.norm(np.cross(xx, yy))
    xh, yh = xx / np.linalg.norm(xx), yy / np.linalg.norm(yy)
    p = w[0] * o + w[1] * h1 + w[2] * h2
    par = [o, h1, h2]
    A = np.array([[1.0, 1.0, 1.0],
                  [float((r - p) @ xh) for r in par],
                  [float((r - p) @ yh) for r in par]])
    lones = []
    geom = [o, h1, h2]
    for wz in (0.5, -0.5):
        tx = np.linalg.solve(A, [0.0, -wz, 0.0])
        ty = np.linalg.solve(A, [0.0, 0.0, -wz])
        lones.append(dict(x=x, y=y, wz=wz, tx=list(tx), ty=list(ty)))
        geom.append(p + wz * zhat)
    geom.append(o + 0.25 * zhat)
    dhh = float(np.linalg.norm(h1 - h2))
    sp = Species("T5R", ["OT", "H", "H", "MW", "MW", "MW"],
                 [0.0, 0.5564, 0.5564, -0.40, -0.40, -0.3128], np.array(geom),
                 bonds=[(0, 1, doh), (0, 2, doh), (1, 2, dhh)])
    sp.dependants = [(3, [(0, w[0]), (1, w[1]), (2, w[2])], "L", lones[0]),
                     (4, [(0, w[0]), (1, w[1]), (2, w[2])], "L", lones[1]),
                     (5, [(0, 1.0), (1, 0.0), (2, 0.0)], "R", dict(wz=0.25))]
    return sp


def ion(name, q=None):
    if q is None:
        q = 1.0 if name == "NA" else -1.0
    return Species(name, [name], [q], np.zeros((1, 3)))


# permanent charges of the Drude water: the SPC/E geometry carrying the
# gas-phase dipole 1.85 D (q_H = 0.3336 e).  With the SPC/E charges (which
# already include the liquid-phase polarization) the added shells polarize
# without bound: O...H contacts close to 1.26 A and the shells run away
# within 60 steps at 298 K even with a fully converged SCF.
DRUDE_WATER_QH = 0.3336


def spce_drude():
    """SPC/E geometry with a Drude shell on the oxygen; permanent charges
    q_H = DRUDE_WATER_QH, q_O = -2 q_H (total site charges; the O core
    carries q_O - q_D)"""
    sp = spce()
    sp.name = "WATD"
    sp.sites = ["OD", "H", "H"]
    sp.charges = [-2 * DRUDE_WATER_QH, DRUDE_WATER_QH, DRUDE_WATER_QH]
    return sp


SPECIES = {"WAT": spce, "NA": lambda: ion("NA"), "CL": lambda: ion("CL"), "WATD": spce_drude,
           "AP": lambda: ion("AP", 1.0), "AM": lambda: ion("AM", -1.0),
           "PRB": lambda: ion("PRB", 0.0), "T4P": tip4p2005, "APV": lambda: ion("APV", 0.8),
           "T5R": water_lone_rowlinson}


@dataclass
class System:
    """Flat site arrays in cook order: species by species, molecule by
    molecule, site by site (the layout of cook's ToInt ``rp`` arrays)."""
    type: np.ndarray       # [ns] int32 LJ type
    q: np.ndarray          # [ns] charge, program units
    mass: np.ndarray       # [ns] mass, program units
    mol: np.ndarray        # [ns] int32 molecule index
    mol_first: np.ndarray  # [nmol+1] first site of each molecule
    cons: np.ndarray       # [nc,2] int32 constrained site pairs (global)
    cons_len: np.ndarray   # [nc] constraint length (A)
    mol_cfirst: np.ndarray # [nmol+1] first constraint of each molecule
    typeE: np.ndarray      # [ntypes] EvdW (K, <=0)
    typeR: np.ndarray      # [ntypes] RvdW (A)
    typeA: np.ndarray      # [ntypes] combining-rule polarizability
    comb_rule: int = 1
    species: list = None
    counts: list = None
    qpol: np.ndarray = None     # [ns] Drude charge (program units) or None
    alphapol: np.ndarray = None # [ns] Drude polarizability volume (A^3) or None
    # dependants (massless sites): site, parents [dep_first[k]:dep_first[k+1]]
    dep_site: np.ndarray = None   # [ndep] int32
    dep_first: np.ndarray = None  # [ndep+1] int32
    dep_parent: np.ndarray = None # [np] int32 (global site indices)
    dep_w: np.ndarray = None      # [np] weights
    dep_type: np.ndarray = None   # [ndep] int32: 0 Middle, 1 Rowlinson, 2 Lone
    dep_par: np.ndarray = None    # [ndep, 13]: wz, x[3], y[3], tx[3], ty[3]

    @property
    def ndep(self):
        return 0 if self.dep_site is None else len(self.dep_site)

    @property
    def polar(self):
        return self.qpol is not None

    @property
    def alpha_qq(self):
        """cook's si->alpha_qq = alphapol/qpol^2 (cook/simdef.c:1008-1010)"""
        a = np.zeros(len(self.type))
        m = self.qpol != 0
        a[m] = self.alphapol[m] / self.qpol[m] ** 2
        return a

    @property
    def ns(self):
        return len(self.type)

    @property
    def nmol(self):
        return len(self.mol_first) - 1


def build_system(species_names, counts):
    E, R, A, _ = type_table()
    tix = {n: i for i, n in enumerate(TYPE_ORDER)}
    typ, q, mass, mol, mfirst, cons, clen, cfirst = [], [], [], [], [0], [], [], [0]
    qpol, apol = [], []
    dsite, dfirst, dpar, dw, dtype, dprm = [], [0], [], [], [], []
    polar = any(t in TYPE_DRUDE for s in species_names for t in SPECIES[s]().sites)
    imol = 0
    for sname, n in zip(species_names, counts):
        sp = SPECIES[sname]()
        for _ in range(n):
            base = len(typ)
            for k, t in enumerate(sp.sites):
                typ.append(tix[t])
                qt = ELECTRON * sp.charges[k]
                ap, cp = TYPE_DRUDE.get(t, (0.0, 0.0))
                qp = cp * ELECTRON
                q.append(qt - qp)          # central charge = total - Drude
                qpol.append(qp)
                apol.append(ap)
                mass.append(ble_type_row(t)[0] / MUNIT)
                mol.append(imol)
            for (i, j, d) in sp.bonds:
                cons.append((base + i, base + j))
                clen.append(d)
            for dep in sp.dependants:
                k, parents = dep[0], dep[1]
                kind = dep[2] if len(dep) > 2 else "M"
                dsite.append(base + k)
                # the weights as cook reads and normalizes them (cook/simdef.c:386-390)
                ws = [float("%.12f" % w) for (_, w) in parents]
                sw = 0.0
                for w in ws:
                    sw += w
                for (pi, _), w in zip(parents, ws):
                    dpar.append(base + pi)
                    dw.append(w / sw)
                dfirst.append(len(dpar))
                dtype.append(DEP_KINDS[kind])
                dprm.append(dep_parameters(kind, dep[3] if len(dep) > 3 else None))
            imol += 1
            mfirst.append(len(typ))
            cfirst.append(len(cons))
    return System(type=np.array(typ, np.int32), q=np.array(q), mass=np.array(mass),
                  mol=np.array(mol, np.int32), mol_first=np.array(mfirst, np.int32),
                  cons=np.array(cons, np.int32).reshape(-1, 2), cons_len=np.array(clen),
                  mol_cfirst=np.array(cfirst, np.int32), typeE=E, typeR=R, typeA=A,
                  comb_rule=1, species=list(species_names), counts=list(counts),
                  qpol=np.array(qpol) if polar else None,
                  alphapol=np.array(apol) if polar else None,
                  dep_site=np.array(dsite, np.int32) if dsite else None,
                  dep_first=np.array(dfirst, np.int32) if dsite else None,
                  dep_parent=np.array(dpar, np.int32) if dsite else None,
                  dep_w=np.array(dw) if dsite else None,
                  dep_type=np.array(dtype, np.int32) if dsite else None,
                  dep_par=np.array(dprm).reshape(-1, 13) if dsite else None)


def ble_text(species_names):
    """The cook force-field (.ble) file of these species (test fixtures);
    with a Drude species the table carries cook's POLAR columns
    alphapol chargepol Esat kappa (cook/simdef.c:638-700)."""
    polar = any(t in TYPE_DRUDE for s in species_names for t in SPECIES[s]().sites)
    lines = ["! force field written by macsimus_gb300.forcefield",
             "nspec=%d" % len(species_names),
             "  nsites=%d  nnbfixes=0  factor14=1  distance14=0  comb_rule=1" % len(TYPE_ORDER),
             "  polar=%d  nparms=0;" % (1 if polar else 0), "", "Lennard-Jones",
             "! i atom mass alpha EvdW[kcal/mol] RvdW[A]" +
             (" alphapol chargepol Esat kappa" if polar else "")]
    for i, n in enumerate(TYPE_ORDER):
        m, ev, rv = ble_type_row(n)
        extra = ""
        if polar:
            ap, cp = TYPE_DRUDE.get(n, (0.0, 0.0))
            extra = " %.12g %.12g 0 0" % (ap, cp)
        lines.append("  %d %-3s %.6f 0 %.12g %.12g%s" % (i, n, m, ev, rv, extra))
    lines += ["", "nbfixes", ""]
    for isp, sname in enumerate(species_names):
        sp = SPECIES[sname]()
        ns = len(sp.sites)
        lines += ["", "species %s" % sname, "", "i=%d  N=0  config=0  water=0" % isp,
                  "ns=%d  nc=%d  nangles=0  ndihedrals=0  nimpropers=0  naromatics=0"
                  % (ns, len(sp.bonds)), "ndependants=%d ;" % len(sp.dependants), "",
                  "sites"]
        for k in range(ns):
            excl = " ".join(str(j) for j in range(k))
            x, y, z = sp.geometry[k]
            lines.append("  %d %-3s %.4f  %.12f %.12f %.12f  %d %s"
                         % (k, sp.sites[k], sp.charges[k], x, y, z, k, excl))
        lines += ["", "bonds"]
        for (i, j, d) in sp.bonds:
            lines.append("  %d %s   %d %s   450  %.15f" % (i, sp.sites[i], j, sp.sites[j], d))
        lines += ["", "angles", "", "dihedrals", "", "impropers", "", "aromatics", "",
                  "dependants"]
        # cook/simdef.c readdependants: kind site name n (parent name weight)...
        # [R: wz | L: x[3] y[3] wz tx[3] ty[3]] e; cook prepends every
        # dependant to its list, so the file lists them last first and cook
        # runs them in the order of sp.dependants
        for dep in reversed(sp.dependants):
            k, parents = dep[0], dep[1]
            kind = dep[2] if len(dep) > 2 else "M"
            line = ("  %s %d %s %d " % (kind, k, sp.sites[k], len(parents)) +
                    " ".join("%d %s %.12f" % (pi, sp.sites[pi], w) for pi, w in parents))
            if kind == "R":
                line += " %.15g" % dep[3]["wz"]
            elif kind == "L":
                e = dep[3]
                line += " " + " ".join("%.15g" % c for c in
                                       list(e["x"]) + list(e["y"]) + [e["wz"]] +
                                       list(e["tx"]) + list(e["ty"]))
            lines.append(line + " e")
        lines += ["", ""]
    return "\n".join(lines) + "\n\n"


def ionic_system(n, sig_p, eps_p, sig_m, eps_m, probe=(3.2, 0.65), masses=(22.9898, 35.453, 39.948)):
    """n/2 cations (+1 e) and n/2 anions (-1 e), LJ spheres (sigma A, epsilon
    kJ/mol), each its own molecule; the type table has a third type, the LJ
    ghost (probe = (sigma, epsilon)) used by Widom insertions, with no site"""
    if n % 2:
        raise ValueError("an equimolar ionic box needs an even number of ions")
    types = [(masses[0], eps_p, sig_p), (masses[1], eps_m, sig_m), (masses[2], probe[1], probe[0])]
    E = np.array([EUNIT_KCAL * _g12(-e / KJ_PER_KCAL) for _, e, _ in types])
    R = np.array([_g12(rvdw_of_sigma(sg)) for _, _, sg in types])
    typ = np.array([0] * (n // 2) + [1] * (n // 2), np.int32)
    q = np.where(typ == 0, ELECTRON, -ELECTRON).astype(np.float64)
    mass = np.array([float("%.6f" % types[t][0]) / MUNIT for t in typ])
    return System(type=typ, q=q, mass=mass, mol=np.arange(n, dtype=np.int32),
                  mol_first=np.arange(n + 1, dtype=np.int32), cons=np.zeros((0, 2), np.int32),
                  cons_len=np.zeros(0), mol_cfirst=np.zeros(n + 1, np.int32), typeE=E, typeR=R,
                  typeA=np.zeros(3), comb_rule=1, species=["ion+", "ion-"],
                  counts=[n // 2, n // 2])
