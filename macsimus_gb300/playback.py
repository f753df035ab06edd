"""cook's playback trajectories: SIMNAME.plb (positions), .vlb (velocities)
and .dlb (Drude positions), written from the device MD state and read back.

File layout (sim/simils.c:1554-1697 openplayback/writeplayback, read by
sim/simils.c:1919-2060 readplayback): a float32 header (ns, -3) -- (ns, -6)
for centred frames, cook's -n4 -- then per frame float32 L[3] followed by ns
float32 triples.  An old-style header (ns, L) with L >= 0 has no per-frame L
(cubic box of side L).  Frames are appended with ``Playback.write`` after the
MD steps, as cook writes one every dt.plb.
"""
import os

import numpy as np

EXT = ("plb", "vlb", "dlb")


class Playback:
    """Open SIMNAME.plb (+ .vlb with ``velocities``, + .dlb with ``drude``)
    for a ForcePath's MD state, as cook's openplayback: ``append`` continues
    existing files after checking their site count; otherwise they are
    (re)created with the header.  ``flags``: cook's -n bits 2 (positions at
    t - h/2) and 4 (centred)."""

    def __init__(self, simname, fp, velocities=False, drude=False, flags=0, append=False):
        if drude and not fp.polar:
            raise ValueError("Drude playback needs a build with Drude charges")
        self.fp = fp
        self.flags = int(flags) & 6
        self.kinds = ["plb"] + (["vlb"] if velocities else []) + (["dlb"] if drude else [])
        self.files = {}
        for k in self.kinds:
            fn = "%s.%s" % (simname, k)
            if append:
                if not os.path.exists(fn):
                    raise FileNotFoundError("%s is about to be appended but does not exist" % fn)
                head = np.fromfile(fn, dtype=np.float32, count=2)
                if len(head) != 2:
                    raise ValueError("%s is too short" % fn)
                if head[0] != fp.ns:
                    raise ValueError("number of sites in %s (ns=%d) does not match ns=%d"
                                     % (fn, int(head[0]), fp.ns))
                self.files[k] = open(fn, "ab")
            else:
                f = open(fn, "wb")
                np.array([fp.ns, -6.0 if self.flags & 4 else -3.0], np.float32).tofile(f)
                self.files[k] = f

    def write(self):
        """append one frame of the current MD state to every open file"""
        for k in self.kinds:
            L, fr = self.fp.playback_frame(k, self.flags if k != "vlb" else 0)
            f = self.files[k]
            L.astype(np.float32).tofile(f)
            fr.astype(np.float32).tofile(f)
            f.flush()

    def close(self):
        for f in self.files.values():
            f.close()
        self.files = {}

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def read_playback(fn):
    """(L [nframes, 3], r [nframes, ns, 3], centred) of a .plb/.vlb/.dlb file"""
    raw = np.fromfile(fn, dtype=np.float32)
    if len(raw) < 2:
        raise ValueError("%s: read header" % fn)
    ns = int(raw[0])
    if raw[1] >= 0:
        fr = raw[2:]
        n = len(fr) // (3 * ns)
        r = fr[:3 * ns * n].reshape(n, ns, 3)
        return np.full((n, 3), raw[1], np.float32), r, False
    if raw[1] not in (-3.0, -6.0):
        raise ValueError("wrong header L=%g in the playback file %s" % (raw[1], fn))
    fr = raw[2:]
    n = len(fr) // (3 * (ns + 1))
    fr = fr[:3 * (ns + 1) * n].reshape(n, ns + 1, 3)
    return fr[:, 0].copy(), fr[:, 1:].copy(), raw[1] == -6.0
