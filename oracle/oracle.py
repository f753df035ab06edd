"""ctypes access to the CPU oracle ``libcookoracle.so`` (TEST INFRASTRUCTURE).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, as the checker.  The product path never does.
"""
import ctypes as C
import os
import subprocess

import math

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libcookoracle.so")


class SS(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("C1q", "C2q", "A", "A4", "Sq", "E4", "E24", "E48", "corr", "eps", "sig")]


class EN(C.Structure):
    _fields_ = [("el", C.c_double), ("lj", C.c_double), ("vir", C.c_double),
                ("Pvir", C.c_double * 6), ("ek", C.c_double), ("er", C.c_double),
                ("eself", C.c_double), ("edip", C.c_double), ("self", C.c_double)]

    def asdict(self):
        return dict(el=self.el, lj=self.lj, vir=self.vir, Pvir=list(self.Pvir), ek=self.ek,
                    er=self.er, eself=self.eself, edip=self.edip, self=self.self)


class SYS(C.Structure):
    _fields_ = [("ns", C.c_int), ("type", C.POINTER(C.c_int)), ("q", C.POINTER(C.c_double)),
                ("mol", C.POINTER(C.c_int)), ("ntypes", C.c_int), ("ss", C.POINTER(SS)),
                ("L", C.c_double * 3), ("cutoff", C.c_double), ("alpha", C.c_double),
                ("kappa", C.c_double), ("epsinf", C.c_double), ("ertab", C.POINTER(C.c_double)),
                ("ntab", C.c_int), ("sgrid", C.c_double), ("qpol", C.POINTER(C.c_double)),
                ("alphaqq", C.POINTER(C.c_double)), ("elcorr", C.c_int)]


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        src = [os.path.join(HERE, n) for n in ("cookoracle.c", "cookoracle.h")]
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(map(os.path.getmtime, src)):
            build()
        L = C.CDLL(LIB)
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        L.orc_setss.argtypes = [C.c_double, C.c_double, C.c_double, C.POINTER(SS)]
        L.orc_combrule.argtypes = [C.c_double] * 6 + [C.c_int, dp, dp]
        L.orc_erfc_ntab.argtypes = [C.c_int, C.c_double, C.c_double]
        L.orc_erfc_build.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, dp, dp]
        L.orc_eru.argtypes = [dp, C.c_double, C.c_double]
        L.orc_eru.restype = C.c_double
        L.orc_erd.argtypes = [dp, C.c_double, C.c_double]
        L.orc_erd.restype = C.c_double
        L.orc_exacterud_sqrt.argtypes = [C.c_double, C.c_double, dp]
        L.orc_exacterud_sqrt.restype = C.c_double
        L.orc_kvectors.argtypes = [dp, dp, C.c_int, ip]
        L.orc_forces.argtypes = [C.POINTER(SYS), dp, dp, C.POINTER(EN), C.c_int]
        L.orc_shake_step.argtypes = [C.c_int, dp, dp, dp, dp, C.c_int, ip, ip, ip, ip, ip, dp,
                                     C.c_double, C.c_double, C.c_double, C.c_int, dp]
        L.orc_shake_step_dp.argtypes = [C.c_int, dp, dp, dp, dp, C.c_int, ip, ip, ip, ip, ip, dp,
                                        C.c_double, C.c_double, C.c_double, C.c_int, dp, dp]
        L.orc_shake_step_meas.argtypes = [C.c_int, dp, dp, dp, dp, C.c_int, ip, ip, ip, ip, ip,
                                          dp, C.c_double, C.c_double, C.c_double, C.c_int, dp,
                                          dp, dp]
        L.orc_selffield.argtypes = [C.POINTER(SYS), dp, dp, C.POINTER(EN), C.c_double]
        L.orc_selffield.restype = C.c_double
        L.orc_aspc_coef.argtypes = [C.c_int, dp, dp]
        u64 = C.c_ulonglong
        L.orc_widom_word.argtypes = [u64, C.c_longlong, C.c_int]
        L.orc_widom_word.restype = u64
        L.orc_widom_sites.argtypes = [u64, C.c_longlong, dp, C.c_int, dp, dp]
        L.orc_einsert.argtypes = [C.POINTER(SYS), dp, C.c_int, ip, dp, dp]
        L.orc_xwidom.argtypes = [C.POINTER(SYS), dp, C.c_int, ip, ip, ip, dp, C.c_double, dp]
        L.orc_xwidom.restype = C.c_double
        L.orc_einsert.restype = C.c_double
        L.orc_widom.argtypes = [C.POINTER(SYS), dp, C.c_int, ip, dp, dp, C.c_longlong, u64,
                                C.c_double, dp, C.c_int]
        L.orc_widom.restype = C.c_double
        L.orc_adjoint.argtypes = [C.POINTER(SYS), dp, dp, dp, dp, dp, dp, dp, dp, dp, dp]
        L.orc_widom_corr.argtypes = [C.POINTER(SYS), C.c_int, ip]
        L.orc_thermostat.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                     C.c_double, C.c_ulonglong, C.c_longlong]
        L.orc_thermostat.restype = C.c_double
        L.orc_widom_corr.restype = C.c_double
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def pair_tables(system, C2):
    """per type pair setss constants (combining rule + smoothing)"""
    L = lib()
    nt = len(system.typeE)
    ss = (SS * (nt * nt))()
    for a in range(nt):
        for b in range(nt):
            eps, sig = C.c_double(), C.c_double()
            L.orc_combrule(system.typeE[a], system.typeR[a], system.typeA[a],
                           system.typeE[b], system.typeR[b], system.typeA[b],
                           system.comb_rule, C.byref(eps), C.byref(sig))
            rc = L.orc_setss(eps.value, sig.value, C2, C.byref(ss[a * nt + b]))
            if rc != 0:
                raise ValueError("setss failed for types %d,%d" % (a, b))
    return ss


def smoothing_derivatives(system, C2):
    """dA/dsigma and dA4/dsigma (sigma of 4 eps[(s/r)^12-(s/r)^6]) of the smooth
    cutoff constants of every type pair, [nt*nt*2], by central differences
    of setss"""
    L = lib()
    nt = len(system.typeE)
    out = np.zeros(nt * nt * 2)
    c6 = 2.0 ** (1.0 / 6.0)
    for a in range(nt):
        for b in range(nt):
            eps, sig = C.c_double(), C.c_double()
            L.orc_combrule(system.typeE[a], system.typeR[a], system.typeA[a],
                           system.typeE[b], system.typeR[b], system.typeA[b],
                           system.comb_rule, C.byref(eps), C.byref(sig))
            if eps.value == 0:
                continue
            h = 1e-5 * sig.value
            sp, sm = SS(), SS()
            L.orc_setss(eps.value, sig.value + h, C2, C.byref(sp))
            L.orc_setss(eps.value, sig.value - h, C2, C.byref(sm))
            # d/d sigma_LJ = c6 d/d r_min
            out[2 * (a * nt + b)] = (sp.A - sm.A) / (2 * h) * c6
            out[2 * (a * nt + b) + 1] = (sp.A4 - sm.A4) / (2 * h) * c6
    return out


def kvectors(Lbox, kappa):
    L = lib()
    Lb = np.ascontiguousarray(Lbox, dtype=np.float64)
    kap = C.c_double(kappa)
    n = L.orc_kvectors(_dp(Lb), C.byref(kap), 0, None)
    kv = np.zeros((n, 3), np.int32)
    kap = C.c_double(kappa)
    L.orc_kvectors(_dp(Lb), C.byref(kap), n, _ip(kv))
    return kv, kap.value


class Oracle:
    """The oracle's view of one system + Ewald parameters."""

    def __init__(self, system, Lbox, cutoff, alpha, kappa, LJcutoff=None, grid=256,
                 rshift=3, rplus=2.5, epsinf=3e33, elcorr=0):
        L = lib()
        self.system = system
        self.L = np.array(Lbox, dtype=np.float64)
        self.ss = pair_tables(system, LJcutoff if LJcutoff else cutoff)
        ntab = L.orc_erfc_ntab(grid, cutoff + rplus, alpha)
        self.tab = np.zeros(6 * ntab)
        sg = C.c_double()
        L.orc_erfc_build(grid, cutoff + rplus, cutoff, alpha, rshift, _dp(self.tab), C.byref(sg))
        self.kv, self.kappa = kvectors(self.L, kappa)
        self.type = np.ascontiguousarray(system.type, np.int32)
        self.q = np.ascontiguousarray(system.q, np.float64)
        self.mol = np.ascontiguousarray(system.mol, np.int32)
        s = SYS()
        s.ns = system.ns
        s.type = _ip(self.type)
        s.q = _dp(self.q)
        s.mol = _ip(self.mol)
        s.ntypes = len(system.typeE)
        s.ss = self.ss
        for k in range(3):
            s.L[k] = self.L[k]
        s.cutoff = cutoff
        s.alpha = alpha
        s.kappa = self.kappa
        s.epsinf = epsinf
        s.elcorr = elcorr
        s.ertab = _dp(self.tab)
        s.ntab = ntab
        s.sgrid = sg.value
        if getattr(system, "polar", False):
            self.qpol = np.ascontiguousarray(system.qpol, np.float64)
            self.alphaqq = np.ascontiguousarray(system.alpha_qq, np.float64)
            s.qpol = _dp(self.qpol)
            s.alphaqq = _dp(self.alphaqq)
        else:
            s.qpol = None
            s.alphaqq = None
        self.polar = getattr(system, "polar", False)
        self.sys = s
        self.sgrid = sg.value
        self.ntab = ntab

    def forces(self, r, measure=True, nthreads=1):
        r = np.ascontiguousarray(r, dtype=np.float64).reshape(-1)
        f = np.zeros_like(r)
        en = EN()
        lib().orc_forces(C.byref(self.sys), _dp(r), _dp(f), C.byref(en) if measure else None,
                         nthreads)
        return f.reshape(-1, 3), (en.asdict() if measure else None)

    def selffield(self, r2, f2, omega, en=None):
        """one Drude iteration: r2/f2 [2ns,3] updated in place; en dict
        (from forces) updated with the self-pair Ewald term, En.self, Pvir"""
        r2 = np.ascontiguousarray(r2, dtype=np.float64)
        f2 = np.ascontiguousarray(f2, dtype=np.float64)
        e = EN()
        if en is not None:
            e.el = en["el"]
            for m in range(6):
                e.Pvir[m] = en["Pvir"][m]
        d = lib().orc_selffield(C.byref(self.sys), _dp(r2.reshape(-1)), _dp(f2.reshape(-1)),
                                C.byref(e), omega)
        if en is not None:
            en = dict(en)
            en["el"] = e.el
            en["self"] = e.self
            en["Pvir"] = list(e.Pvir)
        return r2, f2, en, d

    def shake_step(self, r, r1, f, h, eps=1e-10, omega=0.6, maxit=1000, dp=None, meas=None):
        """leap-frog + SHAKE (dp: added to the unconstrained positions); meas
        (a float64 array of 13) receives En.virc, PTvirc[6] and the kinetic
        tensor En.Pkin[6] before the division by V"""
        s = self.system
        r = np.ascontiguousarray(r, dtype=np.float64).copy().reshape(-1)
        r1 = np.ascontiguousarray(r1, dtype=np.float64).copy().reshape(-1)
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        mass = np.ascontiguousarray(s.mass, np.float64)
        mfirst = np.ascontiguousarray(s.mol_first, np.int32)
        cfirst = np.ascontiguousarray(s.mol_cfirst, np.int32)
        nc = np.ascontiguousarray(np.diff(s.mol_cfirst), np.int32)
        ci = np.ascontiguousarray(s.cons[:, 0], np.int32)
        cj = np.ascontiguousarray(s.cons[:, 1], np.int32)
        bq = np.ascontiguousarray(s.cons_len ** 2, np.float64)
        ek = C.c_double()
        dpa = None if dp is None else np.ascontiguousarray(dp, np.float64).reshape(-1)
        it = lib().orc_shake_step_meas(s.ns, _dp(r), _dp(r1), _dp(f), _dp(mass), s.nmol,
                                       _ip(mfirst), _ip(nc), _ip(cfirst), _ip(ci), _ip(cj),
                                       _dp(bq), h, eps, omega, maxit,
                                       _dp(dpa) if dpa is not None else None, C.byref(ek),
                                       _dp(meas) if meas is not None else None)
        return r.reshape(-1, 3), r1.reshape(-1, 3), it, ek.value


    # ---------------------------------------------------------- adjoint --
    def adjoint(self, r, g=None, C2=None):
        """gradients of E, W and (g = dLoss/dF) a force loss w.r.t. the LJ
        (eps, sigma) of every type pair a<=b and every site charge"""
        s = self.system
        nt = len(s.typeE)
        r = np.ascontiguousarray(r, np.float64).reshape(-1)
        gg = None if g is None else np.ascontiguousarray(g, np.float64).reshape(-1)
        dA = smoothing_derivatives(s, C2 if C2 else self.sys.cutoff)
        E, W = C.c_double(), C.c_double()
        dEp, dWp, dLp = (np.zeros(nt * nt * 2) for _ in range(3))
        dEq, dLq = np.zeros(s.ns), np.zeros(s.ns)
        rc = lib().orc_adjoint(C.byref(self.sys), _dp(r), _dp(gg) if gg is not None else None,
                               _dp(dA), C.byref(E), C.byref(W), _dp(dEp), _dp(dWp), _dp(dLp),
                               _dp(dEq), _dp(dLq))
        if rc:
            raise ValueError("orc_adjoint: polar systems are not supported")
        sh = (nt, nt, 2)
        return dict(E=E.value, W=W.value, dEp=dEp.reshape(sh), dWp=dWp.reshape(sh),
                    dLp=dLp.reshape(sh), dEq=dEq, dLq=dLq)

    # ------------------------------------------------------------ Widom --
    def widom_sites(self, seed, k, geometry):
        g = np.ascontiguousarray(geometry, np.float64).reshape(-1, 3)
        out = np.zeros_like(g)
        lib().orc_widom_sites(seed, k, _dp(self.L), len(g), _dp(g), _dp(out))
        return out

    def einsert(self, r, probe_types, probe_q, positions):
        r = np.ascontiguousarray(r, np.float64).reshape(-1)
        pt = np.ascontiguousarray(probe_types, np.int32)
        pq = np.ascontiguousarray(probe_q, np.float64)
        pp = np.ascontiguousarray(positions, np.float64).reshape(-1)
        return lib().orc_einsert(C.byref(self.sys), _dp(r), len(pt), _ip(pt), _dp(pq), _dp(pp))

    def xwidom(self, r, mols, vtype, vq, T):
        """identity change of the listed molecules to site types vtype and
        charges vq (cook's XWidom): (sum of exp(-dU/T), dU per molecule)"""
        s = self.system
        r = np.ascontiguousarray(r, dtype=np.float64).reshape(-1)
        mols = np.ascontiguousarray(mols, np.int32)
        vtype = np.ascontiguousarray(vtype, np.int32)
        vq = np.ascontiguousarray(vq, np.float64)
        mf = np.ascontiguousarray(s.mol_first, np.int32)
        dU = np.zeros(len(mols))
        tot = lib().orc_xwidom(C.byref(self.sys), _dp(r), len(mols), _ip(mols), _ip(mf),
                               _ip(vtype), _dp(vq), T, _dp(dU))
        return tot, dU

    def widom(self, r, probe_types, probe_q, geometry, n, seed, T, energies=False, nthreads=8):
        """(sum of exp(-U/T), corr, U or None) over n insertions"""
        r = np.ascontiguousarray(r, np.float64).reshape(-1)
        pt = np.ascontiguousarray(probe_types, np.int32)
        pq = np.ascontiguousarray(probe_q, np.float64)
        g = np.ascontiguousarray(geometry, np.float64).reshape(-1)
        U = np.zeros(n) if energies else None
        s = lib().orc_widom(C.byref(self.sys), _dp(r), len(pt), _ip(pt), _dp(pq), _dp(g), n,
                            seed, T, _dp(U) if energies else None, nthreads)
        corr = lib().orc_widom_corr(C.byref(self.sys), len(pt), _ip(pt))
        return s, corr, U


def _dep_kind(system, k):
    t = getattr(system, "dep_type", None)
    return 0 if t is None else int(t[k])


def depend_r(system, r):
    """positions of the dependants from their parents, in table order
    (sim/norm.c:1161-1231, depend_r): linear ("Middle") r_d = sum_p w_p r_p;
    "Rowlinson" r_d = D0 + wz l/|l|, l = (D1 - D0) x (D2 - D0); "Lone"
    r_d = sum_p w_p D_p + wz z/|z|, z = (sum x_p D_p) x (sum y_p D_p);
    returns a copy"""
    r = np.array(r, dtype=np.float64, copy=True)
    for k in range(system.ndep):
        a, b = system.dep_first[k], system.dep_first[k + 1]
        par = system.dep_parent[a:b]
        kind = _dep_kind(system, k)
        if kind == 1:
            wz = system.dep_par[k][0]
            h1 = r[par[1]] - r[par[0]]
            h2 = r[par[2]] - r[par[0]]
            l = np.cross(h1, h2)
            r[system.dep_site[k]] = r[par[0]] + (wz / math.sqrt(l @ l)) * l
        elif kind == 2:
            q = system.dep_par[k]
            d = np.zeros(3)
            xx = np.zeros(3)
            yy = np.zeros(3)
            for c in range(3):
                d += system.dep_w[a + c] * r[par[c]]
                xx += q[1 + c] * r[par[c]]
                yy += q[4 + c] * r[par[c]]
            zz = np.cross(xx, yy)
            r[system.dep_site[k]] = d + (q[0] / math.sqrt(zz @ zz)) * zz
        else:
            r[system.dep_site[k]] = (system.dep_w[a:b, None] * r[par]).sum(0)
    return r


def depend_f(system, f, r=None, virial=False):
    """forces on the dependants added to their parents in table order
    (sim/norm.c:1276-1360, depend_f): linear f_p += w_p f_d; "Rowlinson" the
    force onto D0 and the torque about D0 through forces along l on D1, D2;
    "Lone" f_p += w_p f_d + alpha_p z with alpha_p = fx tx_p + fy ty_p (r:
    the positions, needed by the two out-of-plane kinds); the dependant
    keeps its force, as in cook; returns a copy.  virial=True also returns
    the scalar virial and the virial tensor (xx yy zz yz zx xy) that the two
    out-of-plane kinds add to cook's En.vir and En.Pvir
    (sim/norm.c:1335-1338, 1363-1368; the tensor of Q, F, G is
    Q (G_x F_x, G_y F_y, G_z F_z, G_y F_z, G_z F_x, G_x F_y),
    sim/norm.c:1256-1262)"""
    f = np.array(f, dtype=np.float64, copy=True)
    vir = 0.0
    pv = np.zeros(6)

    def tensor(q, F, G):
        pv[:] += q * np.array([G[0] * F[0], G[1] * F[1], G[2] * F[2],
                               G[1] * F[2], G[2] * F[0], G[0] * F[1]])

    for k in range(system.ndep):
        fd = f[system.dep_site[k]].copy()
        a, b = system.dep_first[k], system.dep_first[k + 1]
        par = system.dep_parent[a:b]
        kind = _dep_kind(system, k)
        if kind == 1:
            h1 = r[par[1]] - r[par[0]]
            h2 = r[par[2]] - r[par[0]]
            l = r[system.dep_site[k]] - r[par[0]]
            M = np.cross(l, fd)
            Mp = np.cross(l, M)
            h1h1, h2h2, h1h2 = h1 @ h1, h2 @ h2, h1 @ h2
            det = (h1h1 * h2h2 - h1h2 * h1h2) * (l @ l)
            a1 = ((Mp @ h1) * h2h2 - (Mp @ h2) * h1h2) / det
            a2 = ((Mp @ h2) * h1h1 - (Mp @ h1) * h1h2) / det
            f[par[0]] += fd - (a1 + a2) * l
            f[par[1]] += a1 * l
            f[par[2]] += a2 * l
            tensor(a1, l, h1)
            tensor(a2, l, h2)
            tensor(-1.0, l, fd)
            vir -= l @ fd
        elif kind == 2:
            q = system.dep_par[k]
            xx = np.zeros(3)
            yy = np.zeros(3)
            for c in range(3):
                xx += q[1 + c] * r[par[c]]
                yy += q[4 + c] * r[par[c]]
            zz = np.cross(xx, yy)
            rr = zz @ zz
            fx = (xx @ fd) / math.sqrt((xx @ xx) * rr)
            fy = (yy @ fd) / math.sqrt((yy @ yy) * rr)
            fz = (zz @ fd) / rr
            rd = r[system.dep_site[k]]
            rr = math.sqrt(rr)
            for c in range(3):
                alpha = fx * q[7 + c] + fy * q[10 + c]
                f[par[c]] += system.dep_w[a + c] * fd + alpha * zz
                tensor(alpha, zz, r[par[c]] - rd)
            vir -= q[0] / rr * fz
            tensor(-q[0] / rr, fd, zz)
        else:
            for qi in range(a, b):
                f[system.dep_parent[qi]] += system.dep_w[qi] * fd
    if virial:
        return f, vir, pv
    return f


def normalize(system, r, L, r0=0.15):
    """cook's normalize(-1) (sim/norm.c:415-444): per molecule and axis, the
    lowest coordinate over the massive sites below r0 shifts the molecule by
    +L, at or above r0 + L by -L; returns a copy"""
    r = np.array(r, dtype=np.float64, copy=True)
    L = np.broadcast_to(np.asarray(L, dtype=np.float64), (3,))
    for n in range(system.nmol):
        a, b = system.mol_first[n], system.mol_first[n + 1]
        heavy = system.mass[a:b] != 0
        lo = r[a:b][heavy].min(axis=0)
        r[a:b] += np.where(lo < r0, L, np.where(lo >= r0 + L, -L, 0.0))
    return r


def bounddr(r1, drmax):
    """cook's bounddr (sim/norm.c:1513-1560): every site's displacement in
    one step longer than drmax scaled to drmax; returns (r1, sites reduced,
    smallest factor)"""
    r1 = np.array(r1, np.float64).reshape(-1, 3)
    vv = (r1 * r1).sum(1)
    big = vv > drmax * drmax
    q = np.sqrt(drmax * drmax / vv[big])
    r1[big] *= q[:, None]
    return r1, int(big.sum()), float(q.min()) if big.any() else 1.0


def remove_drift(system, r1):
    """cook's removedrifts for the momentum bits (sim/norm.c:677-705): the
    mass-weighted mean of r1 subtracted from every site; returns (r1, the
    drift in A per step)"""
    r1 = np.array(r1, np.float64).reshape(-1, 3)
    m = np.asarray(system.mass, np.float64)[:, None]
    v = (m * r1).sum(0) / m.sum()
    return r1 - v, v


def trvp_coef(k):
    """time-reversible velocity predictor of length k (sim/trvpscale.c:31-35;
    J. Chem. Theory Comput. 7, 3596 (2011)): h v(t) ~ sum_j b_j X_j"""
    b = [(2 * k + 1) / (k + 1)]
    for j in range(k):
        b.append(-b[j] * (k - j) / (k + j + 2))
    return b


class NoseHoover:
    """cook's Nose-Hoover thermostat for Verlet + SHAKE (thermostat=2):
    sim/trvpscale.c (predicted velocities of all degrees of freedom from the
    last k <= pred displacements, k growing from 0), sim/verlet.c:22-37
    (p = h^2 f/m + r + r1 - Vfactor v_pred, Vfactor the predicted h dlogs/dt)
    and sim/thermo.c:180-212 (leap-frog of logs with the step's temperature,
    the extended energy of VERLET=3)."""

    def __init__(self, T, tau, nf, h, pred=2):
        self.T, self.tau, self.nf, self.h, self.pred = T, tau, nf, h, pred
        self.k, self.hist, self.lhist = 0, [], []
        self.logs = self.logsv = 0.0
        self.ext = 0.0

    def step(self, orc, r, r1, f, eps=1e-10, omega=0.6):
        h, k = self.h, self.k
        b = trvp_coef(k)
        X = [np.asarray(r1, np.float64)] + self.hist[:k]
        Lx = [self.logsv] + self.lhist[:k]
        vpred = sum(bj * xj for bj, xj in zip(b, X))
        vfactor = sum(bj * lj for bj, lj in zip(b, Lx))
        knew = min(self.pred, k + 1)
        self.hist = [np.array(r1, np.float64)] + self.hist[:knew - 1]
        self.lhist = [self.logsv] + self.lhist[:knew - 1]
        self.k = knew
        rn, r1n, it, ek = orc.shake_step(r, r1, f, h, eps=eps, omega=omega, dp=-vfactor * vpred)
        # En.T of cook: twice the kinetic energy over No.f
        Tk = 2 * ek / self.nf
        ld, lo = self.logsv, self.logs
        self.logsv += h * h * (Tk / self.T - 1) / self.tau ** 2
        self.logs += self.logsv
        self.ext = self.nf * self.T * (lo + (self.tau / h) ** 2 * (ld ** 2 + self.logsv ** 2) / 4)
        return rn, r1n, it, ek


def aspc_coef(k):
    B = np.zeros(k + 2)
    om = C.c_double()
    lib().orc_aspc_coef(k, _dp(B), C.byref(om))
    return B, om.value


def thermostat_factor(kind, kin2, h, nf, T, tau, seed=0, step=0):
    """velocity factor of cook's Berendsen (1) / Bussi (2) thermostat"""
    return lib().orc_thermostat(kind, kin2, h, nf, T, tau, seed, step)


def drude_md(orc, system, r, r1, h, k, niter, nsteps, epsc, omegac, measure=False):
    """ASPC + SCF + SHAKE steps of a Drude box (sim/constrd.c:726-736 with
    sim/pred2.c:26-100 and sim/scf.c): the predictor history restarted from
    r (displacements of cfg[0]) and r1 (of cfg[1]) as cook restarts it, k the
    ASPC length, niter force evaluations + SCF iterations per step.  Returns
    (r, r1, pressure of the last step or None)."""
    ns = system.ns
    hist = [np.zeros((ns, 3)) for _ in range(k + 2)]
    hist[0] = r[ns:].copy()
    hist[k + 1] = r1[ns:].copy()
    hp, kk = 0, 0
    om = 0.6
    r, r1 = r.copy(), r1.copy()
    K2 = k + 2
    press = None
    for step in range(nsteps):
        meas_step = measure and step == nsteps - 1
        B, _ = aspc_coef(kk)
        pred = sum(B[i] * hist[(hp - i) % K2] for i in range(kk + 2))
        if kk < k:
            kk += 1
            om = aspc_coef(kk)[1]
        r2 = np.vstack([r[:ns], pred])
        for it in range(niter):
            last = meas_step and it == niter - 1
            f2, en = orc.forces(r2, measure=last, nthreads=4)
            r2, f2, en, _ = orc.selffield(r2, f2, om, en if last else None)
        hp = (hp + 1) % K2
        hist[hp] = r2[ns:].copy()
        meas = np.zeros(13) if meas_step else None
        rs, r1s, it, ek = orc.shake_step(r2[:ns], r1[:ns], f2[:ns], h, eps=epsc,
                                         omega=omegac / 2, meas=meas)
        if meas_step:
            press = measure_pressure(en, meas, ek, orc.L)
            press["ekin"] = ek
        r = np.vstack([rs, r2[ns:]])
        r1 = np.vstack([r1s, r1[ns:]])
    return r, r1, press


PUNIT = 13806490.0   # Pa per K/A^3 (sim/units.h:103)


def measure_pressure(en, meas, ekin, L):
    """cook's measurePconstraints (sim/constrd.c:115-265) with No.Pkinq = 1:
    en = energies of the step's force evaluation (+ the SCF iteration for
    Drude builds: el, self, vir, Pvir), meas = the 13 sums of shake_step,
    ekin = the kinetic energy.  Returns K/A^3 values: Pvir (+ constraint
    part), Pkin, Ptens = Pvir + Pkin (xx yy zz yz zx xy), P = cook's Pevir,
    and virc, vir (= En.vir after the constraint and electrostatic parts)."""
    V = float(np.prod(L))
    virc = float(meas[0])
    Pvir = (np.asarray(en["Pvir"], float) + np.asarray(meas[1:7])) / V
    Pkin = np.asarray(meas[7:13]) / V
    vir = en["vir"] + virc + en["el"] - 2 * en.get("self", 0.0)
    return dict(virc=virc, vir=vir, Pvir=Pvir, Pkin=Pkin, Ptens=Pvir + Pkin,
                P=(2 * ekin + vir) / (3 * V))
