"""Generate the golden parity fixtures by running the reference MACSIMUS `cook`.

This script is test infrastructure.  It needs the reference binaries built by
``oracle/build_ref.sh`` (they are compiled from the reference sources into
``oracle/_ref/``), writes hand-made force-field (.ble), parameter (.def) and
run (.get) files into a scratch directory, runs cook with ``-v128`` (every
``forces()`` call dumps ``r q f`` per site, sim/simils.c:2259 ``dumpall``)
and stores the dumps as compact ``.npz`` fixtures next to this file.

Reference input formats followed here: force-field tables as parsed by
cook/simdef.c:500-1000 (``readblend``), run data as parsed by
sim/mainget.c:67-256.  Units are cook program units: K, Angstrom, ps, charge
unit = e/408.779826922048 (sim/units.h:101-108); masses in g/mol in the .ble.

usage: python tests/golden/make_golden.py [case ...]
"""
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REFBIN = os.path.join(REPO, "oracle", "_ref")

sys.path.insert(0, REPO)
from macsimus_gb300.forcefield import ble_text  # noqa: E402


CASES = {
    # 216 SPC/E waters, cutoff 9 A, alpha 0.35/A, |n|<=6
    "spce216": dict(binary="cookew", species=["WAT"], N=[216], L=18.6206,
                    cutoff=9.0, alpha=0.35, kn=6, steps=3, h=0.002, epsc=1e-10),
    # 216 SPC/E under cook's Nose-Hoover thermostat (tau.T 0.05 ps, the
    # Verlet+SHAKE form with the time-reversible velocity predictor, k <= 2
    # by the default -p229); playback (-y) and velocity playback (-n1) frames
    # after every step give the initial r1 the dumps lack
    "nose216": dict(binary="cookew", species=["WAT"], N=[216], L=18.6206,
                    cutoff=9.0, alpha=0.35, kn=6, steps=5, h=0.002, epsc=1e-10,
                    options=["-y99999", "-n1"], extra_def=["thermostat=2", "tau.T=0.05"],
                    extra_get=["dt.plb=0.002"]),
    # the 864 SPC/E configuration: L=29.65 A, cutoff 12, alpha 0.26, |n|<=8
    "spce864": dict(binary="cookew", species=["WAT"], N=[864], L=29.65,
                    cutoff=12.0, alpha=0.26, kn=8, steps=2, h=0.002, epsc=1e-10),
    # small brine: 500 SPC/E + 16 Na+ + 16 Cl-, cutoff 10, alpha 0.31, |n|<=7
    "brine532": dict(binary="cookew", species=["WAT", "NA", "CL"], N=[500, 16, 16],
                     L=24.97, cutoff=10.0, alpha=0.31, kn=7, steps=2, h=0.002,
                     epsc=1e-10),
    # 216 Drude waters (SPC/E + Drude shell on O, alpha 1.44 A^3, q_D -1.8 e),
    # ASPC k=2 (-p220) with one SCF iteration per step (scf.eps=-1)
    "drude216": dict(binary="cookpol", species=["WATD"], N=[216], L=18.6206,
                     cutoff=9.0, alpha=0.35, kn=6, steps=6, h=0.001, epsc=1e-10,
                     options=["-p220"], extra_def=["scf.eps=-1"]),
    # 216 TIP4P/2005 waters: the charge site M is a massless linear
    # dependant of O, H, H (cook's depend_r / depend_f)
    # with a playback (-y) and velocity playback (-n1) frame after every step
    "tip4p216": dict(binary="cookew", species=["T4P"], N=[216], L=18.6206,
                     cutoff=9.0, alpha=0.35, kn=6, steps=3, h=0.002, epsc=1e-10,
                     options=["-y99999", "-n1"], extra_get=["dt.plb=0.002"]),
    # 216 rigid waters with two "Lone" (out-of-plane) dependants and one
    # "Rowlinson" dependant each (test model T5R: cook's DEP_L and DEP_R,
    # sim/norm.c:1196-1231, 1304-1360), charged so that they carry force
    "t5r216": dict(binary="cookew", species=["T5R"], N=[216], L=18.6206,
                   cutoff=9.0, alpha=0.35, kn=6, steps=3, h=0.002, epsc=1e-10),
    # the dipole term of Ewald(2) (sim/ewald.c:865-887) on the 216 SPC/E box:
    # isotropic surroundings of dielectric constant 1 (el.epsinf), the
    # Yeh-Berkowitz slab term along z (el.corr=4), and its energy-only
    # form (el.corr=12)
    "dip216eps": dict(binary="cookew", species=["WAT"], N=[216], L=18.6206,
                      cutoff=9.0, alpha=0.35, kn=6, steps=2, h=0.002, epsc=1e-10,
                      extra_def=["el.epsinf=1"], epsinf=1.0, elcorr=0),
    "dip216yb": dict(binary="cookew", species=["WAT"], N=[216], L=18.6206,
                     cutoff=9.0, alpha=0.35, kn=6, steps=2, h=0.002, epsc=1e-10,
                     extra_def=["el.corr=4"], epsinf=3e33, elcorr=4),
    "dip216yb8": dict(binary="cookew", species=["WAT"], N=[216], L=18.6206,
                      cutoff=9.0, alpha=0.35, kn=6, steps=2, h=0.002, epsc=1e-10,
                      extra_def=["el.corr=12"], epsinf=3e33, elcorr=12),
    # cook's step limiter bounddr (sim/norm.c:1513): drmax=-0.02 A (negative:
    # on for any start) reduces the step of the fast sites after every step
    "bounddr216": dict(binary="cookew", species=["WAT"], N=[216], L=18.6206,
                       cutoff=9.0, alpha=0.35, kn=6, steps=4, h=0.002, epsc=1e-10,
                       extra_get=["drmax=-0.02"], drmax=0.02),
    # Widom insertions of a neutral LJ probe (sigma 3.2 A, epsilon 0.65
    # kJ/mol) into 250 + 250 LJ ions of charge +-1 e, L = 37 A (reduced
    # density 0.5 at sigma 3.7 A), cutoff 10, alpha 0.31, |n|<=8; 1e7
    # insertions into the configuration of the last force evaluation
    "widom500": dict(binary="cookwidom", species=["AP", "AM", "PRB"], N=[250, 250, 0],
                     L=37.0, cutoff=10.0, alpha=0.31, kn=8, steps=1, h=0.002, epsc=1e-10,
                     extra_def=["corr=1"], extra_get=["widom.sp=2", "widom.n=10000000"]),
    # identity change AP -> APV (sigma 3.3 -> 3.4 A, epsilon 0.5 -> 0.55
    # kJ/mol, charge +1 -> +0.8 e) of every cation of the same box
    # (sim/simmeas.c XWidom, cook/widom.c Eidchange)
    "xwidom500": dict(binary="cookwidom", species=["AP", "AM", "APV"], N=[250, 250, 0],
                      L=37.0, cutoff=10.0, alpha=0.31, kn=8, steps=1, h=0.002, epsc=1e-10,
                      extra_get=["widom.spreal=0", "widom.sp=2"]),
}


def def_text(c):
    lines = []
    for i, n in enumerate(c["N"]):
        lines.append("N[%d]=%d" % (i, n))
    L = c["L"]
    lines += ["L[0]=%.10g L[1]=%.10g L[2]=%.10g" % (L, L, L),
              "cutoff=%.10g LJcutoff=%.10g" % (c["cutoff"], c["cutoff"]),
              "noint=1", "h=%.10g" % c["h"], "T=298",
              "el.test=0 el.alpha=%.10g el.kappa=%.12g" % (c["alpha"], (c["kn"] + 1e-6) / L),
              "epsc=%.3g" % c["epsc"], "corr=0"] + c.get("extra_def", []) + [";", ""]
    return "\n".join(lines)


def get_text(c):
    return "\n".join(['init="crystal"', "no=%d" % c["steps"]] + c.get("extra_get", []) +
                     [";", ""])


def parse_dump(path):
    with open(path) as f:
        head = f.readline().split()
        ns = int(head[0])
        L = [float(x) for x in f.readline().split()[:3]]
        rows = []
        for _ in range(ns):
            t = f.readline().split()
            if "rDrude[]" in t:
                # r q rDrude qDrude f fDrude mol site (POLAR dump)
                rows.append([float(x) for x in t[:14]] + [int(t[14]), int(t[15])])
            else:
                rows.append([float(x) for x in t[:7]] + [int(t[7]), int(t[8])])
    a = np.array(rows)
    if a.shape[1] == 16:
        return dict(L=np.array(L), r=a[:, 0:3], q=a[:, 3], rD=a[:, 4:7], qD=a[:, 7],
                    f=a[:, 8:11], fD=a[:, 11:14], mol=a[:, 14].astype(np.int32),
                    site=a[:, 15].astype(np.int32))
    return dict(L=np.array(L), r=a[:, 0:3], q=a[:, 3], f=a[:, 4:7],
                mol=a[:, 7].astype(np.int32), site=a[:, 8].astype(np.int32))


def run_case(name, c, keep=None):
    binary = os.path.join(REFBIN, c["binary"])
    if not os.path.exists(binary):
        raise SystemExit("missing %s: run oracle/build_ref.sh first" % binary)
    wd = keep or tempfile.mkdtemp(prefix="golden_")
    os.makedirs(wd, exist_ok=True)
    with open(os.path.join(wd, "ff.ble"), "w") as f:
        f.write(ble_text(c["species"]))
    with open(os.path.join(wd, "sim.def"), "w") as f:
        f.write(def_text(c))
    with open(os.path.join(wd, "sim.get"), "w") as f:
        f.write(get_text(c))
    p = subprocess.run([binary, "ff.ble", "sim", "-v128"] + c.get("options", []), cwd=wd,
                       stdin=subprocess.DEVNULL, capture_output=True, text=True, timeout=600)
    if p.returncode != 0:
        raise SystemExit("%s failed:\n%s" % (name, p.stdout[-3000:]))
    prt = open(os.path.join(wd, "sim.prt")).read()
    dumps = []
    i = 0
    while os.path.exists(os.path.join(wd, "sim.%d.dump" % i)):
        dumps.append(parse_dump(os.path.join(wd, "sim.%d.dump" % i)))
        i += 1
    m = re.findall(r"En\.pot=(\S+) En\.kin=(\S+) En\.tot=(\S+)", prt)
    m2 = re.search(r"Q->N=(\d+)", prt)
    m3 = re.search(r"omegac=(\S+) \(optimized\)", prt)
    meta = dict(case=name, params=c, ndumps=len(dumps),
                Epot_last=float(m[-1][0]), Ekin_last=float(m[-1][1]), Etot_last=float(m[-1][2]),
                QN=int(m2.group(1)) if m2 else None,
                omegac=float(m3.group(1)) if m3 else None,
                species=c["species"], N=c["N"])
    mw = re.search(r"mu = (\S+) \+- \S+ K \(raw value without cutoff correction\)", prt)
    if mw and "widom.spreal" in get_text(c):
        # identity change: cook prints mu = -T ln <exp(-dU/T)> over the molecules
        mc = re.search(r"corr = (\S+)/V = (\S+)", prt)
        meta["xwidom"] = dict(mu_raw_K=float(mw.group(1)), corr=float(mc.group(1)))
    elif mw:
        mc = re.search(r"corr = (\S+)/V = (\S+)", prt)
        mk = re.search(r"mu = (\S+) \+- \S+ kT \(corrected\)", prt)
        meta["widom"] = dict(mu_raw_K=float(mw.group(1)), corr=float(mc.group(1)),
                             mu_kT=float(mk.group(1)),
                             n=int(re.search(r"widom\.n=(\d+)", get_text(c)).group(1)))
    # playback files (sim/simils.c:1554-1697): float32 header (ns, -3), then
    # per frame L[3] and ns positions (.plb) or velocities (.vlb)
    for ext in ("plb", "vlb"):
        fn = os.path.join(wd, "sim." + ext)
        if os.path.exists(fn):
            raw = np.fromfile(fn, dtype=np.float32)
            ns = int(raw[0])
            assert raw[1] == -3
            fr = raw[2:].reshape(-1, ns + 1, 3)
            dumps[0][ext + "_L"] = fr[:, 0].copy()
            dumps[0][ext + "_r"] = fr[:, 1:].copy()
    if keep is None:
        shutil.rmtree(wd)
    return dumps, meta


# Energy-conservation runs: per-step Etot of cook's own integrator, read from
# the table that cook prints every measurement cycle (noint=1: every step;
# sim/maincps.c, columns t/ps Tkin/K Epot/K Etot/K).  The 864-water box of
# the SPC/E configuration equilibrates from cook's crystal start under the
# Berendsen thermostat (tau.T 0.1 ps, 1500 steps), then runs 5000 NVE steps.
ENERGY_CASES = {
    "nve864": dict(binary="cookewP1", species=["WAT"], N=[864], L=29.65, cutoff=12.0,
                   alpha=0.26, kn=8, h=0.002, epsc=1e-10,
                   sweeps=[dict(thermostat="Berendsen", tau_T=0.1, steps=1500),
                           dict(thermostat="none", steps=5000)]),
}


def run_energy_case(name, c):
    binary = os.path.join(REFBIN, c["binary"])
    if not os.path.exists(binary):
        raise SystemExit("missing %s: run oracle/build_ref.sh first" % binary)
    wd = tempfile.mkdtemp(prefix="golden_")
    with open(os.path.join(wd, "ff.ble"), "w") as f:
        f.write(ble_text(c["species"]))
    with open(os.path.join(wd, "sim.def"), "w") as f:
        f.write(def_text(dict(c, steps=0)))
    sw = []
    for i, w in enumerate(c["sweeps"]):
        lines = ['init="crystal"'] if i == 0 else []
        lines.append('thermostat="%s"' % w["thermostat"])
        if "tau_T" in w:
            lines.append("tau.T=%g" % w["tau_T"])
        lines += ["no=%d" % w["steps"], ";"]
        sw.append("\n".join(lines))
    with open(os.path.join(wd, "sim.get"), "w") as f:
        f.write("\n".join(sw) + "\n")
    env = dict(os.environ, NSLOTS=str(min(os.cpu_count() or 1, 16)))
    p = subprocess.run([binary, "ff.ble", "sim"], cwd=wd, stdin=subprocess.DEVNULL, env=env,
                       capture_output=True, text=True, timeout=3600)
    if p.returncode != 0:
        raise SystemExit("%s failed:\n%s" % (name, p.stdout[-3000:]))
    rows = []
    for line in open(os.path.join(wd, "sim.prt")):
        m = re.match(r"\s+(\d+\.\d{3})\s+(\S+)\s+(-?\d+)\s+(-?\d+\.\d+)\s", line)
        if m:
            rows.append([float(m.group(k)) for k in (1, 2, 3, 4)])
    a = np.array(rows)
    nsteps = sum(w["steps"] for w in c["sweeps"])
    assert a.shape[0] == nsteps, (a.shape, nsteps)
    shutil.rmtree(wd)
    n0 = c["sweeps"][0]["steps"]
    # t of the first NVE step, then per step the printed Tkin (K) and Etot (K)
    meta = dict(case=name, params=c, t0=a[n0, 0], Tkin=a[n0:, 1].tolist(),
                Etot=a[n0:, 3].tolist())
    with open(os.path.join(HERE, name + ".json"), "w") as f:
        json.dump(meta, f, sort_keys=True)
    print("wrote %s: %d NVE steps" % (name, len(meta["Etot"])))


# NVE drift with error bars that resolve a factor of two: four runs of the
# 864-water box from independent crystal starts (cook option -z: the seed of
# its random velocities), each 1500 Berendsen steps then 25000 NVE steps.
# Stored per run: block means of the printed per-step Etot over 50 steps and
# the mean Tkin.  (cook's own regression of Etot(t), LRAdd("Etot") at
# sim/maincps.c:276-277, runs only under the Berendsen and stochastic
# thermostats, so the NVE drift is taken from the printed Etot.)
NVE_ENSEMBLES = {
    "nve864x4": dict(binary="cookewP1", species=["WAT"], N=[864], L=29.65, cutoff=12.0,
                     alpha=0.26, kn=8, h=0.002, epsc=1e-10, seeds=[11, 12, 13, 14],
                     equil=1500, steps=25000, block=50, threads=2),
}


def run_nve_ensemble(name, c):
    binary = os.path.join(REFBIN, c["binary"])
    if not os.path.exists(binary):
        raise SystemExit("missing %s: run oracle/build_ref.sh first" % binary)
    procs = []
    for seed in c["seeds"]:
        wd = tempfile.mkdtemp(prefix="golden_")
        with open(os.path.join(wd, "ff.ble"), "w") as f:
            f.write(ble_text(c["species"]))
        with open(os.path.join(wd, "sim.def"), "w") as f:
            f.write(def_text(dict(c, steps=0)))
        with open(os.path.join(wd, "sim.get"), "w") as f:
            f.write('init="crystal"\nthermostat="Berendsen"\ntau.T=0.1\nno=%d\n;\n'
                    'thermostat="none"\nno=%d\n;\n' % (c["equil"], c["steps"]))
        env = dict(os.environ, NSLOTS=str(c["threads"]))
        procs.append((seed, wd, subprocess.Popen([binary, "ff.ble", "sim", "-z%d" % seed],
                                                 cwd=wd, stdin=subprocess.DEVNULL, env=env,
                                                 stdout=subprocess.DEVNULL,
                                                 stderr=subprocess.DEVNULL)))
    runs = []
    for seed, wd, p in procs:
        if p.wait() != 0:
            raise SystemExit("%s seed %d failed" % (name, seed))
        rows = []
        prt = open(os.path.join(wd, "sim.prt")).read()
        for line in prt.splitlines():
            m = re.match(r"\s+(\d+\.\d{3})\s+(\S+)\s+(-?\d+)\s+(-?\d+\.\d+)\s", line)
            if m:
                rows.append([float(m.group(k)) for k in (1, 2, 3, 4)])
        a = np.array(rows)
        assert a.shape[0] == c["equil"] + c["steps"], a.shape
        nve = a[c["equil"]:]
        b = c["block"]
        nb = len(nve) // b
        runs.append(dict(seed=seed, t0=nve[0, 0], Tkin_mean=float(nve[:, 1].mean()),
                         Etot_block=nve[:nb * b, 3].reshape(nb, b).mean(1).tolist()))
        shutil.rmtree(wd)
    meta = dict(case=name, params=c, runs=runs)
    with open(os.path.join(HERE, name + ".json"), "w") as f:
        json.dump(meta, f, sort_keys=True)
    print("wrote %s: %d runs" % (name, len(runs)))


# Resume parity through cook's .cfg files (sim/simils.c savecfg/loadcfg):
# run A from cook's crystal start writes sim.cfg; run B continues from that
# file (init="cont"); run C continues from a file that
# macsimus_gb300.cfgfile writes: A's state with r1 = r(t) - r(t-h) scaled by
# c["r1_scale"].  Stored: A's file as it is, the final cfg[0] / cfg[1] of B
# and C, and the SHA-256 of the file written for C.
RESUME_CASES = {
    "resume216": dict(binary="cookew", species=["WAT"], N=[216], L=18.6206, cutoff=9.0,
                      alpha=0.35, kn=6, h=0.002, epsc=1e-10, steps_a=4, steps_b=3,
                      r1_scale=0.5),
    # the same with 216 Drude waters (POLAR build, ASPC k=2 + one SCF
    # iteration): cfg[0] and cfg[1] hold 2 ns vectors, the Drude
    # displacements after the sites
    "resume_drude216": dict(binary="cookpol", species=["WATD"], N=[216], L=18.6206,
                            cutoff=9.0, alpha=0.35, kn=6, h=0.001, epsc=1e-10, steps_a=4,
                            steps_b=3, r1_scale=0.5, options=["-p220"],
                            extra_def=["scf.eps=-1"]),
}


def run_resume_case(name, c):
    import hashlib
    from macsimus_gb300 import cfgfile
    binary = os.path.join(REFBIN, c["binary"])
    if not os.path.exists(binary):
        raise SystemExit("missing %s: run oracle/build_ref.sh first" % binary)
    wd = tempfile.mkdtemp(prefix="golden_")
    with open(os.path.join(wd, "ff.ble"), "w") as f:
        f.write(ble_text(c["species"]))
    with open(os.path.join(wd, "sim.def"), "w") as f:
        f.write(def_text(dict(c, steps=0)))

    def run(init, steps):
        with open(os.path.join(wd, "sim.get"), "w") as f:
            f.write('init="%s"\nno=%d\n;\n' % (init, steps))
        p = subprocess.run([binary, "ff.ble", "sim"] + c.get("options", []), cwd=wd,
                           stdin=subprocess.DEVNULL, capture_output=True, text=True, timeout=600)
        if p.returncode != 0:
            raise SystemExit("%s failed:\n%s" % (name, p.stdout[-3000:]))
        return cfgfile.read_cfg(os.path.join(wd, "sim.cfg"))

    run("crystal", c["steps_a"])
    a_bytes = open(os.path.join(wd, "sim.cfg"), "rb").read()
    with open(os.path.join(HERE, name + "_a.cfg"), "wb") as f:
        f.write(a_bytes)
    b = run("cont", c["steps_b"])
    a = cfgfile.read_cfg(os.path.join(HERE, name + "_a.cfg"))
    r, r1 = a["cfg"][0]["rp"], a["cfg"][1]["rp"]
    w = cfgfile.cfg_with_state(a, r, r1 * c["r1_scale"])
    cfgfile.write_cfg(os.path.join(wd, "sim.cfg"), w)
    sha = hashlib.sha256(open(os.path.join(wd, "sim.cfg"), "rb").read()).hexdigest()
    cc = run("cont", c["steps_b"])
    shutil.rmtree(wd)
    np.savez_compressed(os.path.join(HERE, name + ".npz"),
                        rB=b["cfg"][0]["rp"], r1B=b["cfg"][1]["rp"],
                        rC=cc["cfg"][0]["rp"], r1C=cc["cfg"][1]["rp"])
    meta = dict(case=name, params=c, sha256_written=sha, tB=b["t"], tC=cc["t"],
                omegac=None)
    with open(os.path.join(HERE, name + ".json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("wrote %s" % name)


# Pressure of one measured step (cook's measurePconstraints, sim/constrd.c:
# 115-265, with the constraint virial of sim/virc.c): builds with
# PRESSURETENSOR 7 (full tensor).  Run A from cook's crystal start writes
# sim.cfg after steps_a steps; run B appends one step from that file
# (init="append": no earlier statistics loaded) with -v134: -v128 dumps the
# forces, -v2|-v4 print every statistic of the step (its only sample) with
# 9 significant digits.  Stored: A's file and B's printed values.
PRESSURE_CASES = {
    "press_spce216": dict(binary="cookewpt", species=["WAT"], N=[216], L=18.6206, cutoff=9.0,
                          alpha=0.35, kn=6, h=0.002, epsc=1e-10, steps_a=4),
    "press_tip4p216": dict(binary="cookewpt", species=["T4P"], N=[216], L=18.6206,
                           cutoff=9.0, alpha=0.35, kn=6, h=0.002, epsc=1e-10, steps_a=4),
    "press_drude216": dict(binary="cookpolpt", species=["WATD"], N=[216], L=18.6206,
                           cutoff=9.0, alpha=0.35, kn=6, h=0.001, epsc=1e-10, steps_a=4,
                           options=["-p220"], extra_def=["scf.eps=-1"]),
    # the Rowlinson and Lone dependants' own virial and tensor terms
    # (sim/norm.c:1335-1337, 1363-1368)
    "press_t5r216": dict(binary="cookewpt", species=["T5R"], N=[216], L=18.6206,
                         cutoff=9.0, alpha=0.35, kn=6, h=0.002, epsc=1e-10, steps_a=4),
}


def run_pressure_case(name, c):
    binary = os.path.join(REFBIN, c["binary"])
    if not os.path.exists(binary):
        raise SystemExit("missing %s: run oracle/build_ref.sh first" % binary)
    wd = tempfile.mkdtemp(prefix="golden_")
    with open(os.path.join(wd, "ff.ble"), "w") as f:
        f.write(ble_text(c["species"]))
    with open(os.path.join(wd, "sim.def"), "w") as f:
        f.write(def_text(dict(c, steps=0)))

    def run(init, steps, opts):
        with open(os.path.join(wd, "sim.get"), "w") as f:
            f.write('init="%s"\nno=%d\n;\n' % (init, steps))
        p = subprocess.run([binary, "ff.ble", "sim"] + c.get("options", []) + opts, cwd=wd,
                           stdin=subprocess.DEVNULL, capture_output=True, text=True, timeout=600)
        if p.returncode != 0:
            raise SystemExit("%s failed:\n%s" % (name, p.stdout[-3000:]))

    run("crystal", c["steps_a"], [])
    with open(os.path.join(wd, "sim.cfg"), "rb") as f:
        a_bytes = f.read()
    with open(os.path.join(HERE, name + "_a.cfg"), "wb") as f:
        f.write(a_bytes)
    os.remove(os.path.join(wd, "sim.sta"))
    run("append", 1, ["-v134"])
    stats = {}
    for line in open(os.path.join(wd, "sim.prt")):
        m = re.match(r"#\s*(\S+)\s+-\s+-\s+1 =(.+)=$", line.rstrip())
        if m:
            stats[m.group(2)] = float(m.group(1))
    d0 = parse_dump(os.path.join(wd, "sim.0.dump"))
    m3 = re.search(r"omegac=(\S+) \(optimized\)", open(os.path.join(wd, "sim.prt")).read())
    shutil.rmtree(wd)
    arrays = dict(r=d0["r"], f=d0["f"])
    if "rD" in d0:
        arrays.update(rD=d0["rD"], fD=d0["fD"])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
    meta = dict(case=name, params=c, stats=stats, omegac=float(m3.group(1)) if m3 else None)
    with open(os.path.join(HERE, name + ".json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("wrote %s: %d printed statistics" % (name, len(stats)))


def save_case(name, dumps, meta):
    arrays = {}
    d0 = dumps[0]
    arrays["q"] = d0["q"]
    arrays["mol"] = d0["mol"]
    arrays["site"] = d0["site"]
    arrays["L"] = d0["L"]
    arrays["r"] = np.stack([d["r"] for d in dumps])
    arrays["f"] = np.stack([d["f"] for d in dumps])
    for k in ("plb_L", "plb_r", "vlb_L", "vlb_r"):
        if k in d0:
            arrays[k] = d0[k]
    if "rD" in d0:
        arrays["qD"] = d0["qD"]
        arrays["rD"] = np.stack([d["rD"] for d in dumps])
        arrays["fD"] = np.stack([d["fD"] for d in dumps])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
    with open(os.path.join(HERE, name + ".json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("wrote %s: %d dumps, %d sites" % (name, len(dumps), len(d0["q"])))


def main(argv):
    names = argv or (list(CASES) + list(ENERGY_CASES) + list(RESUME_CASES) +
                     list(PRESSURE_CASES) + list(NVE_ENSEMBLES))
    for n in names:
        if n in NVE_ENSEMBLES:
            run_nve_ensemble(n, NVE_ENSEMBLES[n])
            continue
        if n in PRESSURE_CASES:
            run_pressure_case(n, PRESSURE_CASES[n])
            continue
        if n in ENERGY_CASES:
            run_energy_case(n, ENERGY_CASES[n])
            continue
        if n in RESUME_CASES:
            run_resume_case(n, RESUME_CASES[n])
            continue
        dumps, meta = run_case(n, CASES[n])
        save_case(n, dumps, meta)


if __name__ == "__main__":
    main(sys.argv[1:])
