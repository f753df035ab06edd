"""GB300 force path for MACSIMUS cook, host-side mirror of cook's interface.

The compute lives in ``libmacgpu.so`` (hand-written sm_103a CUDA behind the C
ABI declared in ``include/macgpu.h``).  This module only marshals arrays:

* ``ForcePath.forces(r, measure)``  <->  cook ``forces(B,A)`` (cook/forces.c:93)
* ``ForcePath.ewald(r)``            <->  cook ``Ewald(1,..)`` + ``Ewald(2,..)``
                                        (sim/ewald.c:258)
* ``ForcePath.md_steps(n)``         <->  cook's step loop around ``Shake()``
                                        (sim/main.c:1511, sim/constrd.c:622)

There is no CPU fallback: without the built library every call raises.
"""
import ctypes as C
import os

import numpy as np

from . import forcefield  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "_build", "libmacgpu.so")

MG_FP64, MG_MIXED = 0, 1
STATUS = {0: "MG_OK", 1: "MG_ERR_ARG", 2: "MG_ERR_CUDA", 3: "MG_ERR_SHAKE",
          4: "MG_ERR_NONFINITE", 5: "MG_ERR_SETUP", 6: "MG_ERR_SIZE", 7: "MG_ERR_SCF",
          8: "MG_ERR_LIST"}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class MGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS.get(code, code), msg))
        self.code = code


class Topology(C.Structure):
    _fields_ = [("ns", C.c_int), ("nmol", C.c_int), ("mol_first", _ip), ("site_type", _ip),
                ("charge", _dp), ("mass", _dp), ("ntypes", C.c_int), ("type_EvdW", _dp),
                ("type_RvdW", _dp), ("type_alpha", _dp), ("comb_rule", C.c_int), ("nc", C.c_int),
                ("cons", _ip), ("cons_len", _dp), ("mol_cfirst", _ip), ("chargepol", _dp),
                ("alphapol", _dp), ("ndep", C.c_int), ("dep_site", _ip), ("dep_first", _ip),
                ("dep_parent", _ip), ("dep_w", _dp), ("dep_type", _ip), ("dep_par", _dp)]


class Params(C.Structure):
    _fields_ = [("L", C.c_double * 3), ("cutoff", C.c_double), ("LJcutoff", C.c_double),
                ("alpha", C.c_double), ("kappa", C.c_double), ("grid", C.c_int),
                ("rshift", C.c_int), ("rplus", C.c_double), ("epsinf", C.c_double),
                ("precision", C.c_int), ("h", C.c_double), ("epsc", C.c_double),
                ("omegac", C.c_double), ("shake_maxit", C.c_int),
                ("cells_per_cutoff", C.c_int), ("aspc_k", C.c_int), ("scf_iter", C.c_int),
                ("scf_omega", C.c_double), ("minqq", C.c_double), ("skin", C.c_double),
                ("nl_every", C.c_int), ("kspace_ctas_per_sm", C.c_int), ("pair_variant", C.c_int),
                ("thermostat", C.c_int), ("T", C.c_double), ("tau_T", C.c_double),
                ("thermo_f", C.c_double), ("seed", C.c_ulonglong), ("box_rmin", C.c_double),
                ("no_normalize", C.c_int), ("kspace_engine", C.c_int),
                ("nose_pred", C.c_int), ("dipole_corr", C.c_int), ("drmax", C.c_double),
                ("drift_step", C.c_int),
                ("kspace_serial", C.c_int)]


class Energy(C.Structure):
    _fields_ = [("el", C.c_double), ("lj", C.c_double), ("vir", C.c_double),
                ("Pvir", C.c_double * 6), ("ek", C.c_double), ("er", C.c_double),
                ("eself", C.c_double), ("edip", C.c_double), ("self", C.c_double),
                ("ekin", C.c_double), ("virc", C.c_double), ("Pkin", C.c_double * 6),
                ("Ptens", C.c_double * 6), ("P", C.c_double)]
    _tensors = ("Pvir", "Pkin", "Ptens")

    def asdict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in self._tensors}
        for k in self._tensors:
            d[k] = list(getattr(self, k))
        return d


class AdjointOut(C.Structure):
    _fields_ = [("E", C.c_double), ("W", C.c_double), ("dE_pair", _dp), ("dW_pair", _dp),
                ("dL_pair", _dp), ("dE_dq", _dp), ("dL_dq", _dp)]


class Probe(C.Structure):
    _fields_ = [("ns", C.c_int), ("site_type", _ip), ("charge", _dp), ("geometry", _dp)]


class WidomResult(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("sum", "raw", "corr", "factor", "widom", "mu")]

    def asdict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def library():
    """Load libmacgpu.so (it must have been built: macsimus_gb300/build.py)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise RuntimeError("libmacgpu.so is not built (run python macsimus_gb300/build.py)")
        L = C.CDLL(LIBPATH)
        vp = C.c_void_p
        L.mg_create.argtypes = [C.POINTER(Topology), C.POINTER(Params), _ip]
        L.mg_create.restype = vp
        L.mg_destroy.argtypes = [vp]
        L.mg_last_error.argtypes = [vp]
        L.mg_last_error.restype = C.c_char_p
        L.mg_kappa.argtypes = [vp]
        L.mg_kappa.restype = C.c_double
        L.mg_nkvec.argtypes = [vp]
        L.mg_last_launches.argtypes = [vp]
        L.mg_forces.argtypes = [vp, _dp, _dp, C.c_int, C.POINTER(Energy)]
        L.mg_forces_device.argtypes = [vp, vp, vp, C.c_int, C.POINTER(Energy)]
        L.mg_ewald.argtypes = [vp, _dp, _dp, _dp]
        L.mg_md_set_state.argtypes = [vp, _dp, _dp]
        L.mg_md_get_state.argtypes = [vp, _dp, _dp]
        L.mg_playback_frame.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_float)]
        _fp = C.POINTER(C.c_float)
        L.mg_tc_selftest.argtypes = [_fp, _fp, _fp, C.c_int, C.c_int]
        L.mg_xwidom.argtypes = [vp, C.c_int, _ip, _ip, _dp, C.c_double,
                                C.POINTER(WidomResult), _dp]
        L.mg_md_steps.argtypes = [vp, C.c_int, C.POINTER(Energy)]
        L.mg_selffield.argtypes = [vp, _dp, _dp, C.c_double, C.c_int, C.POINTER(Energy)]
        L.mg_set_stream.argtypes = [vp, vp]
        L.mg_set_overlap.argtypes = [vp, C.c_int]
        L.mg_thermostat_factor.argtypes = [vp]
        L.mg_thermostat_factor.restype = C.c_double
        L.mg_nose_state.argtypes = [vp, _dp]
        L.mg_set_graph.argtypes = [vp, C.c_int]
        L.mg_batch_fused.argtypes = [vp]
        L.mg_batch_profile.argtypes = [vp, C.c_int, _dp]
        L.mg_bounddr_report.argtypes = [vp, C.POINTER(C.c_longlong), _dp]
        L.mg_remove_drift.argtypes = [vp, _dp]
        L.mg_profile_enable.argtypes = [vp, C.c_int]
        L.mg_profile_reset.argtypes = [vp]
        L.mg_profile_entry.argtypes = [vp, C.c_int, C.POINTER(C.c_char_p), _dp,
                                       C.POINTER(C.c_long)]
        L.mg_probe_fp32_tflops.argtypes = [_dp]
        L.mg_autotune.argtypes = [C.POINTER(Topology), C.POINTER(Params), _dp, C.c_int, _dp]
        L.mg_adjoint.argtypes = [vp, _dp, _dp, C.POINTER(AdjointOut)]
        L.mg_widom.argtypes = [vp, C.POINTER(Probe), C.c_longlong, C.c_ulonglong, C.c_double,
                               C.POINTER(WidomResult), _dp]
        L.mg_batch_create.argtypes = [C.c_int, C.POINTER(Topology), C.POINTER(Params), C.c_int,
                                      _ip]
        L.mg_batch_create.restype = vp
        L.mg_batch_destroy.argtypes = [vp]
        L.mg_batch_last_error.argtypes = [vp]
        L.mg_batch_last_error.restype = C.c_char_p
        L.mg_batch_box.argtypes = [vp, C.c_int]
        L.mg_batch_box.restype = vp
        L.mg_batch_last_launches.argtypes = [vp]
        L.mg_batch_md_steps.argtypes = [vp, C.c_int, C.POINTER(Energy)]
        L.mg_batch_widom.argtypes = [vp, C.POINTER(Probe), C.c_int, C.c_longlong, C.c_ulonglong,
                                     C.c_double, C.POINTER(WidomResult)]
        L.mg_ewald_kspace_noalloc.argtypes = [vp, vp, C.c_int, _dp, C.c_double, C.c_double, vp,
                                              _dp, vp]
        _lib = L
    return _lib


def autotune(system, L, cutoff, alpha, kappa, r, nrep=3, **kw):
    """the fastest (cells_per_cutoff, kspace_ctas_per_sm, pair_variant,
    kspace_serial) for this box and configuration (mg_autotune), with the
    timings (3x3 grid x split, the 8 cell-kernel pair variants, the group
    kernel and its two half-shell forms at cdiv 1..3, the chosen variant
    with the Ewald chain concurrent and serial)"""
    t, p, keep = describe(system, L, cutoff, alpha, kappa, **kw)
    ms = np.full(28, -1.0)
    rr = _arr(r, np.float64).reshape(-1)
    rc = library().mg_autotune(C.byref(t), C.byref(p), rr.ctypes.data_as(_dp), int(nrep),
                               ms.ctypes.data_as(_dp))
    if rc:
        raise MGError(rc, "mg_autotune failed")
    return dict(cells_per_cutoff=p.cells_per_cutoff, kspace_ctas_per_sm=p.kspace_ctas_per_sm,
                pair_variant=p.pair_variant, kspace_serial=p.kspace_serial,
                ms=ms[:9].reshape(3, 3), ms_pair=ms[9:17], ms_group=ms[17:20],
                ms_half=ms[20:23], ms_serial=ms[23:25], ms_half_t=ms[25:28])


def fp32_peak_tflops():
    """measured FP32 FMA throughput of the current device (TFLOP/s)"""
    t = C.c_double()
    rc = library().mg_probe_fp32_tflops(C.byref(t))
    if rc:
        raise MGError(rc, "FP32 probe failed")
    return t.value


def _arr(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def describe(system, L, cutoff, alpha, kappa, precision="mixed", LJcutoff=None, grid=256,
             rshift=3, rplus=2.5, epsinf=3e33, h=0.002, epsc=1e-7, omegac=1.2, shake_maxit=1000,
             cells_per_cutoff=0, aspc_k=2, scf_iter=1, scf_omega=0.6, minqq=1.0, skin=0.0,
             nl_every=50, kspace_ctas_per_sm=0, pair_variant=0, thermostat=0, T=298.0,
             tau_T=0.1, thermo_f=0.0, seed=0, box_rmin=0.0, normalize=True, kspace_engine=0,
             nose_pred=2, dipole_corr=0, drmax=0.0, drift_step=False, kspace_serial=0):
    """(mg_topology, mg_params, arrays to keep alive) of one box"""
    keep = []

    def ip(a):
        a = _arr(a, np.int32)
        keep.append(a)
        return a.ctypes.data_as(_ip)

    def dp(a):
        a = _arr(a, np.float64)
        keep.append(a)
        return a.ctypes.data_as(_dp)

    t = Topology()
    t.ns = system.ns
    t.nmol = system.nmol
    t.mol_first = ip(system.mol_first)
    t.site_type = ip(system.type)
    t.charge = dp(system.q)
    t.mass = dp(system.mass)
    t.ntypes = len(system.typeE)
    t.type_EvdW = dp(system.typeE)
    t.type_RvdW = dp(system.typeR)
    t.type_alpha = dp(system.typeA)
    t.comb_rule = system.comb_rule
    t.nc = len(system.cons_len)
    t.cons = ip(system.cons.reshape(-1))
    t.cons_len = dp(system.cons_len)
    t.mol_cfirst = ip(system.mol_cfirst)
    if getattr(system, "ndep", 0):
        t.ndep = system.ndep
        t.dep_site = ip(system.dep_site)
        t.dep_first = ip(system.dep_first)
        t.dep_parent = ip(system.dep_parent)
        t.dep_w = dp(system.dep_w)
        if system.dep_type is not None and (system.dep_type != 0).any():
            t.dep_type = ip(system.dep_type)
            t.dep_par = dp(system.dep_par)
    else:
        t.ndep = 0
    if getattr(system, "polar", False):
        t.chargepol = dp(system.qpol)
        t.alphapol = dp(system.alphapol)
    else:
        t.chargepol = None
        t.alphapol = None
    p = Params()
    Lb = np.broadcast_to(np.asarray(L, dtype=np.float64), (3,))
    for k in range(3):
        p.L[k] = float(Lb[k])
    p.cutoff = cutoff
    p.LJcutoff = LJcutoff if LJcutoff else cutoff
    p.alpha = alpha
    p.kappa = kappa
    p.grid = grid
    p.rshift = rshift
    p.rplus = rplus
    p.epsinf = epsinf
    p.precision = MG_MIXED if precision == "mixed" else MG_FP64
    p.h = h
    p.epsc = epsc
    p.omegac = omegac
    p.shake_maxit = shake_maxit
    p.cells_per_cutoff = cells_per_cutoff
    p.aspc_k = aspc_k
    p.scf_iter = scf_iter
    p.scf_omega = scf_omega
    p.minqq = minqq
    p.skin = skin
    p.nl_every = nl_every
    p.kspace_ctas_per_sm = kspace_ctas_per_sm
    p.pair_variant = pair_variant
    p.thermostat = {"none": 0, "berendsen": 1, "bussi": 2,
                    "nose": 3}.get(thermostat, thermostat) or 0
    p.T = T
    p.tau_T = tau_T
    p.thermo_f = thermo_f
    p.seed = seed
    p.box_rmin = box_rmin
    p.no_normalize = 0 if normalize else 1
    p.kspace_engine = int(kspace_engine)
    p.nose_pred = int(nose_pred)
    p.dipole_corr = int(dipole_corr)
    p.drmax = float(drmax)
    p.drift_step = 1 if drift_step else 0
    p.kspace_serial = int(kspace_serial)
    return t, p, keep


class ForcePath:
    """One box on the current GPU: topology + Ewald/LJ parameters."""

    def __init__(self, system, L, cutoff, alpha, kappa, precision="mixed", LJcutoff=None,
                 grid=256, rshift=3, rplus=2.5, epsinf=3e33, h=0.002, epsc=1e-7, omegac=1.2,
                 shake_maxit=1000, cells_per_cutoff=0, aspc_k=2, scf_iter=1, scf_omega=0.6,
                 minqq=1.0, skin=0.0, nl_every=50, kspace_ctas_per_sm=0, pair_variant=0,
                 thermostat=0, T=298.0, tau_T=0.1, thermo_f=0.0, seed=0, box_rmin=0.0,
                 normalize=True, kspace_engine=0, nose_pred=2, dipole_corr=0, drmax=0.0,
                 drift_step=False, kspace_serial=0):
        lib = library()
        self.system = system
        self.ns = system.ns
        t, p, self._keep = describe(system, L, cutoff, alpha, kappa, precision=precision,
                                    LJcutoff=LJcutoff, grid=grid, rshift=rshift, rplus=rplus,
                                    epsinf=epsinf, h=h, epsc=epsc, omegac=omegac,
                                    shake_maxit=shake_maxit, cells_per_cutoff=cells_per_cutoff,
                                    aspc_k=aspc_k, scf_iter=scf_iter, scf_omega=scf_omega,
                                    minqq=minqq, skin=skin, nl_every=nl_every,
                                    kspace_ctas_per_sm=kspace_ctas_per_sm,
                                    pair_variant=pair_variant, thermostat=thermostat, T=T,
                                    tau_T=tau_T, thermo_f=thermo_f, seed=seed,
                                    box_rmin=box_rmin, normalize=normalize,
                                    kspace_engine=kspace_engine, nose_pred=nose_pred,
                                    dipole_corr=dipole_corr, drmax=drmax,
                                    drift_step=drift_step, kspace_serial=kspace_serial)
        self.polar = getattr(system, "polar", False)
        Lb = np.broadcast_to(np.asarray(L, dtype=np.float64), (3,))
        st = C.c_int(0)
        self._ctx = lib.mg_create(C.byref(t), C.byref(p), C.byref(st))
        if not self._ctx:
            raise MGError(st.value, "mg_create failed")
        self._owned = True
        self.precision = precision
        self.thermostat = p.thermostat
        self.L = np.array(Lb)
        self.kappa = lib.mg_kappa(self._ctx)
        self.nkvec = lib.mg_nkvec(self._ctx)

    @classmethod
    def _borrow(cls, ctx, system, L, precision, owner):
        """a view of a context owned by a Batch (not destroyed by close())"""
        fp = cls.__new__(cls)
        fp._ctx = ctx
        fp._owned = False
        fp._owner = owner
        fp.system = system
        fp.ns = system.ns
        fp.polar = getattr(system, "polar", False)
        fp.precision = precision
        fp.L = np.array(np.broadcast_to(np.asarray(L, dtype=np.float64), (3,)))
        fp.kappa = library().mg_kappa(ctx)
        fp.nkvec = library().mg_nkvec(ctx)
        return fp

    def close(self):
        if getattr(self, "_ctx", None):
            if getattr(self, "_owned", True):
                library().mg_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise MGError(rc, library().mg_last_error(self._ctx).decode())

    @property
    def launches(self):
        return library().mg_last_launches(self._ctx)

    def forces(self, r, measure=False):
        """cook forces(B,A): returns (f [ns,3], energy dict or None)."""
        r = _arr(r, np.float64).reshape(-1)
        f = np.empty_like(r)
        en = Energy()
        self._check(library().mg_forces(self._ctx, r.ctypes.data_as(_dp), f.ctypes.data_as(_dp),
                                        int(measure), C.byref(en)))
        return f.reshape(-1, 3), (en.asdict() if measure else None)

    def forces_device(self, r_ptr, f_ptr, measure=False):
        """forces on device arrays (raw CUDA pointers, e.g. tensor.data_ptr())."""
        en = Energy()
        self._check(library().mg_forces_device(self._ctx, C.c_void_p(r_ptr), C.c_void_p(f_ptr),
                                               int(measure), C.byref(en)))
        return en.asdict() if measure else None

    def ewald(self, r):
        """k-space forces and energy (k + self terms), cook Ewald passes 1+2."""
        r = _arr(r, np.float64).reshape(-1)
        f = np.zeros_like(r)
        e = C.c_double()
        self._check(library().mg_ewald(self._ctx, r.ctypes.data_as(_dp), f.ctypes.data_as(_dp),
                                       C.byref(e)))
        return f.reshape(-1, 3), e.value

    def selffield(self, r, f, omega, en=None):
        """cook selffield(): one SCF iteration; r, f with 2*ns vectors.
        Returns (r, f, en) with en the energies of the forces call updated"""
        r = _arr(r, np.float64).reshape(-1).copy()
        f = _arr(f, np.float64).reshape(-1).copy()
        e = Energy()
        if en is not None:
            for k, v in en.items():
                if k in Energy._tensors:
                    for m in range(6):
                        getattr(e, k)[m] = v[m]
                else:
                    setattr(e, k, v)
        self._check(library().mg_selffield(self._ctx, r.ctypes.data_as(_dp),
                                           f.ctypes.data_as(_dp), omega, int(en is not None),
                                           C.byref(e)))
        return r.reshape(-1, 3), f.reshape(-1, 3), (e.asdict() if en is not None else None)

    def md_set_state(self, r, r1):
        r = _arr(r, np.float64).reshape(-1)
        r1 = _arr(r1, np.float64).reshape(-1)
        self._check(library().mg_md_set_state(self._ctx, r.ctypes.data_as(_dp),
                                              r1.ctypes.data_as(_dp)))

    def md_get_state(self, out=None):
        """(r, r1) of the device MD state; out = (r, r1): contiguous float64
        arrays (e.g. pinned host buffers) to copy into instead of new ones"""
        nv = 3 * self.ns * (2 if self.polar else 1)
        if out is None:
            r, r1 = np.empty(nv), np.empty(nv)
        else:
            r, r1 = out
            for a in (r, r1):
                if a.dtype != np.float64 or a.size != nv or not a.flags.c_contiguous:
                    raise ValueError("out arrays must be contiguous float64 of %d values" % nv)
        self._check(library().mg_md_get_state(self._ctx, r.ctypes.data_as(_dp),
                                              r1.ctypes.data_as(_dp)))
        return r.reshape(-1, 3), r1.reshape(-1, 3)

    def md_load_cfg(self, path):
        """MD state from cook's SIMNAME.cfg (loadcfg, sim/simils.c:1150):
        cfg[0] = r(t), cfg[1] = r(t) - r(t-h); returns the parsed file"""
        from . import cfgfile
        c = cfgfile.read_cfg(path)
        if c["polar"] != self.polar:
            raise cfgfile.CfgError("POLAR file for a non-polar box or the reverse")
        r, r1 = cfgfile.state_from_cfg(c, self.ns)
        self.md_set_state(r, r1)
        return c

    def md_save_cfg(self, path, template, t=None, Etot=None):
        """the device MD state as cook's SIMNAME.cfg (savecfg,
        sim/simils.c:1445); the other records (options, species, box,
        thermostat) come from template, a parsed .cfg of the same system;
        a Nose-Hoover context also writes logs and h dlogs/dt"""
        from . import cfgfile
        r, r1 = self.md_get_state()
        nose = self.nose_state()[:2] if getattr(self, "thermostat", 0) == 3 else None
        cfgfile.write_cfg(path, cfgfile.cfg_with_state(template, r, r1, t=t, Etot=Etot,
                                                       nose=nose))

    def xwidom(self, mols, vtype, vcharge, T, energies=False):
        """cook's XWidom identity change of the listed molecules into sites of
        types vtype and charges vcharge (program units) in the configuration
        of the last force evaluation: dict(sum, raw, mu) (+ dU per molecule)"""
        mols = np.ascontiguousarray(mols, np.int32)
        vt = np.ascontiguousarray(vtype, np.int32)
        vq = np.ascontiguousarray(vcharge, np.float64)
        res = WidomResult()
        dU = np.zeros(len(mols)) if energies else None
        self._check(library().mg_xwidom(self._ctx, len(mols), mols.ctypes.data_as(_ip),
                                        vt.ctypes.data_as(_ip), vq.ctypes.data_as(_dp), float(T),
                                        C.byref(res), dU.ctypes.data_as(_dp) if energies else None))
        out = dict(sum=res.sum, raw=res.raw, mu=res.mu)
        if energies:
            out["dU"] = dU
        return out

    def playback_frame(self, what="plb", flags=0):
        """(L[3], float32 [ns, 3]) of the MD state as cook writes it into
        SIMNAME.plb ("plb": r), .vlb ("vlb": r1/h) or .dlb ("dlb": r + the
        Drude offset); flags are cook's -n bits 2 (r - r1/2) and 4 (r - L/2)"""
        w = {"plb": 0, "vlb": 1, "dlb": 2}[what]
        fr = np.empty(3 * (self.ns + 1), np.float32)
        self._check(library().mg_playback_frame(self._ctx, w, int(flags),
                                                fr.ctypes.data_as(C.POINTER(C.c_float))))
        fr = fr.reshape(-1, 3)
        return fr[0].copy(), fr[1:]

    def thermostat_factor(self):
        """velocity factor of the last thermostat call"""
        return library().mg_thermostat_factor(self._ctx)

    def remove_drift(self):
        """cook's removedrifts (momentum) on the MD state; returns the removed
        drift velocity, A/ps"""
        v = np.zeros(3)
        self._check(library().mg_remove_drift(self._ctx, v.ctypes.data_as(_dp)))
        return v

    def bounddr_report(self):
        """(sites whose step was reduced, smallest factor) since the last
        report: cook's bounddr with drmax"""
        n, q = C.c_longlong(), C.c_double()
        self._check(library().mg_bounddr_report(self._ctx, C.byref(n), C.byref(q)))
        return n.value, q.value

    def nose_state(self):
        """Nose-Hoover (thermostat="nose"): (logs, h dlogs/dt, the thermostat's
        part of the conserved energy of the last step, K)"""
        st = (C.c_double * 3)()
        self._check(library().mg_nose_state(self._ctx, st))
        return tuple(st)

    def set_overlap(self, on):
        """FP32 path: k-space chain concurrent with the r-space chain (default on)"""
        self._check(library().mg_set_overlap(self._ctx, 1 if on else 0))

    def set_graph(self, on):
        """MD steps as one replayed CUDA graph each (default) or kernel by kernel"""
        self._check(library().mg_set_graph(self._ctx, 1 if on else 0))

    def set_stream(self, stream_handle):
        """run on a caller's CUDA stream (e.g. torch.cuda.current_stream().cuda_stream)"""
        self._check(library().mg_set_stream(self._ctx, C.c_void_p(stream_handle or None)))

    def profile(self, on=True):
        self._check(library().mg_profile_enable(self._ctx, int(on)))

    def profile_reset(self):
        self._check(library().mg_profile_reset(self._ctx))

    def profile_read(self):
        """{kernel name: (total ms, launches)} recorded while profiling was on"""
        out = {}
        i = 0
        while True:
            name = C.c_char_p()
            ms = C.c_double()
            cnt = C.c_long()
            if library().mg_profile_entry(self._ctx, i, C.byref(name), C.byref(ms), C.byref(cnt)):
                break
            out[name.value.decode()] = (ms.value, cnt.value)
            i += 1
        return out

    def md_steps(self, n, measure=True):
        en = Energy()
        self._check(library().mg_md_steps(self._ctx, int(n), C.byref(en) if measure else None))
        return en.asdict() if measure else None

    def adjoint(self, r, g=None):
        """gradients of E, W = LJ sum r.f + E_el and (g = dLoss/dF, [ns,3]) of
        a force loss w.r.t. the LJ (eps, sigma) of every type pair a <= b
        ([nt,nt,2]) and every site charge ([ns]); FP64 contexts"""
        nt = len(self.system.typeE)
        r = _arr(r, np.float64).reshape(-1)
        gg = None if g is None else _arr(g, np.float64).reshape(-1)
        dEp, dWp, dLp = (np.zeros(nt * nt * 2) for _ in range(3))
        dEq, dLq = np.zeros(self.ns), np.zeros(self.ns)
        out = AdjointOut(0.0, 0.0, dEp.ctypes.data_as(_dp), dWp.ctypes.data_as(_dp),
                         dLp.ctypes.data_as(_dp), dEq.ctypes.data_as(_dp), dLq.ctypes.data_as(_dp))
        self._check(library().mg_adjoint(self._ctx, r.ctypes.data_as(_dp),
                                         gg.ctypes.data_as(_dp) if gg is not None else None,
                                         C.byref(out)))
        sh = (nt, nt, 2)
        return dict(E=out.E, W=out.W, dEp=dEp.reshape(sh), dWp=dWp.reshape(sh),
                    dLp=dLp.reshape(sh), dEq=dEq, dLq=dLq)

    def widom(self, site_types, geometry=None, charges=None, n=100000, seed=1, T=298.0,
              energies=False):
        """Widom insertions of a ghost molecule (cook's Einsert + Widom) into
        the configuration of the last force evaluation; returns a dict with
        sum, raw, corr, factor, widom, mu (K) and, with energies=True, the
        insertion energies U [n] (K)"""
        st = _arr(site_types, np.int32).reshape(-1)
        g = _arr(np.zeros((len(st), 3)) if geometry is None else geometry, np.float64).reshape(-1)
        q = None if charges is None else _arr(charges, np.float64).reshape(-1)
        pr = Probe(len(st), st.ctypes.data_as(_ip), q.ctypes.data_as(_dp) if q is not None else None,
                   g.ctypes.data_as(_dp))
        res = WidomResult()
        U = np.zeros(int(n)) if energies else None
        self._check(library().mg_widom(self._ctx, C.byref(pr), int(n), int(seed), float(T),
                                       C.byref(res), U.ctypes.data_as(_dp) if energies else None))
        out = res.asdict()
        if energies:
            out["U"] = U
        return out


class Batch:
    """Independent boxes on the current GPU, stepped together: one captured
    CUDA graph per MD step of all boxes, one kernel launch for the Widom
    insertions of all boxes.  boxes: list of dicts with the ForcePath
    arguments (system, L, cutoff, alpha, kappa, and keywords)."""

    def __init__(self, boxes, precision="mixed", lanes=16):
        lib = library()
        self.nbox = len(boxes)
        tops = (Topology * self.nbox)()
        pars = (Params * self.nbox)()
        self._keep = []
        self.systems = []
        for i, b in enumerate(boxes):
            b = dict(b)
            system = b.pop("system")
            t, p, keep = describe(system, b.pop("L"), b.pop("cutoff"), b.pop("alpha"),
                                  b.pop("kappa"), precision=precision, **b)
            tops[i] = t
            pars[i] = p
            self._keep.append(keep)
            self.systems.append(system)
        st = C.c_int(0)
        self._b = lib.mg_batch_create(self.nbox, tops, pars, int(lanes), C.byref(st))
        if not self._b:
            raise MGError(st.value, "mg_batch_create failed")
        self.precision = precision
        self.box = [ForcePath._borrow(lib.mg_batch_box(self._b, i), self.systems[i],
                                      [pars[i].L[0], pars[i].L[1], pars[i].L[2]], precision, self)
                    for i in range(self.nbox)]

    def _check(self, rc):
        if rc != 0:
            raise MGError(rc, library().mg_batch_last_error(self._b).decode())

    @property
    def launches(self):
        return library().mg_batch_last_launches(self._b)

    @property
    def fused(self):
        """True once MD steps run as one launch per kernel over all boxes"""
        return bool(library().mg_batch_fused(self._b))

    PROFILE_STAGES = ("cell_list", "pair", "phase_tc", "ewald_sk", "ewald_sk_reduce",
                      "ewald_kforce", "shake")

    def profile(self, nrep=5):
        """nrep further MD steps of the fused batch timed stage by stage:
        {stage: ms per step} (mg_batch_profile)"""
        ms = np.zeros(7)
        self._check(library().mg_batch_profile(self._b, int(nrep), ms.ctypes.data_as(_dp)))
        return dict(zip(self.PROFILE_STAGES, ms.tolist()))

    def md_steps(self, n, measure=True):
        en = (Energy * self.nbox)()
        self._check(library().mg_batch_md_steps(self._b, int(n), en if measure else None))
        return [e.asdict() for e in en] if measure else None

    def widom(self, site_types, geometry=None, charges=None, n=100000, seed=1, T=298.0):
        """the same ghost inserted n times into every box (box i uses the
        stream of seed + i * 0x632BE59BD9B4E019); list of result dicts"""
        st = _arr(site_types, np.int32).reshape(-1)
        g = _arr(np.zeros((len(st), 3)) if geometry is None else geometry, np.float64).reshape(-1)
        q = None if charges is None else _arr(charges, np.float64).reshape(-1)
        pr = Probe(len(st), st.ctypes.data_as(_ip), q.ctypes.data_as(_dp) if q is not None else None,
                   g.ctypes.data_as(_dp))
        out = (WidomResult * self.nbox)()
        self._check(library().mg_batch_widom(self._b, C.byref(pr), 0, int(n), int(seed), float(T),
                                             out))
        return [o.asdict() for o in out]

    def close(self):
        if getattr(self, "_b", None):
            for fp in self.box:
                fp._ctx = None
            library().mg_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
