"""cook's configuration file SIMNAME.cfg: read and write.

cook saves its state with ``savecfg`` (sim/simils.c:1445-1517) and loads it
with ``loadcfg`` (sim/simils.c:1150-1410) through the record file of
gen/varfile.c: every record is ``<int4 size><size bytes><int4 checksum>``,
the checksum being 0x4A4B plus the sum of the data bytes (gen/varfile.c:61),
a record of size 0 ends the file, followed by an int4 time key
(``KeyClose``, gen/varfile.c:119).  The records of a .cfg, in order:

  1. ``cfgkey`` (int4; 1, + 2 for POLAR builds, sim/simils.c:953)
  2. the 32 option values of the run (int4 each, options -a .. -z and more)
  3. ``nspec`` (int4), then per species ``{int N; int ns}`` (sim/simils.h:28)
  4. key records ``{int key; int intval; double vecval[3]}``:
     key 1: No.N, (t, h, En.tot); key 2: No.s, box.L; key 4: thermostat,
     (sigvdW, tau.T, tau.P); key 5 (SLAB builds): cleave; key 17 (POLAR):
     tau.dip
  5. cfg[0] .. cfg[m-1] (m = option -m, 2 for Verlet/SHAKE), each the whole
     ``ToInt`` struct of sim/simglob.h:307-315: int size, int dep, double
     logs, double lambda[3], double offdiag[3], double rp[ns][3] (POLAR:
     2 ns vectors, the Drude displacements after the sites).  For the
     Verlet/SHAKE integrator cfg[0] holds r(t) and cfg[1] r(t) - r(t-h); the
     Nose variable logs and h dlogs/dt sit in the logs fields.

The layout is little-endian with 8-byte reals, as cook writes it on the
machines it runs on.
"""
import struct

import numpy as np

VARSUM0 = 0x4A4B
REC_FMT = "<ii3d"          # struct rec_s
REC_SIZE = struct.calcsize(REC_FMT)
HEAD_DOUBLES = 7           # logs, lambda[3], offdiag[3] (RPOFFSET)


class CfgError(ValueError):
    pass


def _records(raw):
    """(list of record payloads, time key) of a varfile byte string"""
    recs, off = [], 0
    while True:
        if off + 4 > len(raw):
            raise CfgError("truncated record header at byte %d" % off)
        (size,) = struct.unpack_from("<i", raw, off)
        off += 4
        if size == 0:
            break
        if size < 0 or off + size + 4 > len(raw):
            raise CfgError("bad record size %d at byte %d" % (size, off - 4))
        data = raw[off:off + size]
        off += size
        (chk,) = struct.unpack_from("<i", raw, off)
        off += 4
        if (VARSUM0 + sum(data)) & 0xFFFFFFFF != chk & 0xFFFFFFFF:
            raise CfgError("checksum mismatch in record %d" % len(recs))
        recs.append(data)
    key = struct.unpack_from("<i", raw, off)[0] if off + 4 <= len(raw) else 0
    return recs, key


def _record(data):
    s = (VARSUM0 + sum(data)) & 0xFFFFFFFF
    if s >= 1 << 31:
        s -= 1 << 32
    return struct.pack("<i", len(data)) + bytes(data) + struct.pack("<i", s)


def read_cfg(path):
    """Parse a cook .cfg; returns a dict with cfgkey, options (32 ints),
    species [(N, ns)], keys {key: (intval, (v0, v1, v2))}, t, h, Etot, L,
    polar, and cfg: a list of dicts (size, dep, logs, lambda, offdiag,
    rp [n, 3] float64), plus timekey."""
    raw = open(path, "rb").read()
    recs, timekey = _records(raw)
    if len(recs) < 5:
        raise CfgError("too few records (%d)" % len(recs))
    (cfgkey,) = struct.unpack("<i", recs[0])
    if not cfgkey & 1:
        raise CfgError("old (<V2.7) configuration format")
    options = list(struct.unpack("<32i", recs[1]))
    (nspec,) = struct.unpack("<i", recs[2])
    sp = struct.unpack("<%di" % (2 * nspec), recs[3])
    species = [(sp[2 * i], sp[2 * i + 1]) for i in range(nspec)]
    keys, i = {}, 4
    while i < len(recs) and len(recs[i]) == REC_SIZE:
        k, iv, v0, v1, v2 = struct.unpack(REC_FMT, recs[i])
        keys[k] = (iv, (v0, v1, v2))
        i += 1
    cfgs = []
    for data in recs[i:]:
        size, dep = struct.unpack_from("<ii", data, 0)
        if size != len(data) or (size - 8) % 8:
            raise CfgError("configuration record of %d bytes says size %d" % (len(data), size))
        vals = np.frombuffer(data, dtype="<f8", offset=8)
        cfgs.append(dict(size=size, dep=dep, logs=float(vals[0]), lam=vals[1:4].copy(),
                         offdiag=vals[4:7].copy(), rp=vals[7:].reshape(-1, 3).copy()))
    if not cfgs:
        raise CfgError("no configuration record")
    out = dict(cfgkey=cfgkey, options=options, species=species, keys=keys, cfg=cfgs,
               timekey=timekey, polar=bool(cfgkey & 2))
    if 1 in keys:
        out["N"] = keys[1][0]
        out["t"], out["h"], out["Etot"] = keys[1][1]
    if 2 in keys:
        out["ns"] = keys[2][0]
        out["L"] = list(keys[2][1])
    return out


def write_cfg(path, c):
    """Write the dict of read_cfg (possibly with new cfg arrays, t, h, Etot,
    L) back in cook's format; a file read and written unchanged comes out
    byte for byte the same."""
    keys = dict(c["keys"])
    if "N" in c or "t" in c:
        iv, v = keys.get(1, (0, (0.0, 0.0, 0.0)))
        keys[1] = (c.get("N", iv), (c.get("t", v[0]), c.get("h", v[1]), c.get("Etot", v[2])))
    if "L" in c or "ns" in c:
        iv, v = keys.get(2, (0, (0.0, 0.0, 0.0)))
        keys[2] = (c.get("ns", iv), tuple(c.get("L", v)))
    out = [_record(struct.pack("<i", c["cfgkey"])),
           _record(struct.pack("<32i", *c["options"])),
           _record(struct.pack("<i", len(c["species"]))),
           _record(struct.pack("<%di" % (2 * len(c["species"])),
                               *[x for s in c["species"] for x in s]))]
    for k in c["keys"]:      # the order of the file read (savecfg's order)
        iv, v = keys[k]
        out.append(_record(struct.pack(REC_FMT, k, iv, *v)))
    for k in keys:
        if k not in c["keys"]:
            iv, v = keys[k]
            out.append(_record(struct.pack(REC_FMT, k, iv, *v)))
    for g in c["cfg"]:
        rp = np.ascontiguousarray(g["rp"], dtype="<f8").reshape(-1)
        vals = np.concatenate([[g["logs"]], np.asarray(g["lam"], "<f8"),
                               np.asarray(g["offdiag"], "<f8"), rp]).astype("<f8")
        size = 8 + 8 * len(vals)
        out.append(_record(struct.pack("<ii", size, g.get("dep", 0)) + vals.tobytes()))
    out.append(struct.pack("<i", 0) + struct.pack("<i", c.get("timekey", 0)))
    with open(path, "wb") as f:
        f.write(b"".join(out))


def state_from_cfg(c, ns):
    """(r, r1) of the Verlet/SHAKE integrator: cfg[0]->rp and cfg[1]->rp,
    ns sites (POLAR files: 2 ns vectors each, sites then Drude displacements)"""
    if len(c["cfg"]) < 2:
        raise CfgError("the file holds %d configurations, Verlet needs 2" % len(c["cfg"]))
    r, r1 = c["cfg"][0]["rp"], c["cfg"][1]["rp"]
    n = 2 * ns if c["polar"] else ns
    if r.shape[0] != n or r1.shape[0] != n:
        raise CfgError("the file holds %d vectors per configuration, expected %d"
                       % (r.shape[0], n))
    return r.copy(), r1.copy()


def cfg_with_state(c, r, r1, t=None, Etot=None, nose=None):
    """A copy of the parsed file c with cfg[0]->rp = r and cfg[1]->rp = r1
    (and optionally t, En.tot and the Nose variables (logs, h dlogs/dt))"""
    d = dict(c)
    d["keys"] = dict(c["keys"])
    d["cfg"] = [dict(g) for g in c["cfg"]]
    for g, a in zip(d["cfg"][:2], (r, r1)):
        a = np.asarray(a, np.float64)
        if a.shape != g["rp"].shape:
            raise CfgError("state of shape %s for a record of %s" % (a.shape, g["rp"].shape))
        g["rp"] = a.copy()
        g["dep"] = 0
    if t is not None:
        d["t"] = t
    if Etot is not None:
        d["Etot"] = Etot
    if nose is not None:
        d["cfg"][0]["logs"], d["cfg"][1]["logs"] = float(nose[0]), float(nose[1])
    return d
