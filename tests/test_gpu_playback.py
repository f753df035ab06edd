"""Playback frames from the device MD state against cook's own .plb/.vlb
files (written by cook -y -n1 beside the tip4p216 dumps; sim/simils.c
writeplayback), and the file layout round trip."""
import numpy as np
import pytest

import macsimus_gb300 as M
from golden_cases import load
from macsimus_gb300.playback import Playback, read_playback

pytestmark = pytest.mark.gpu

F32 = np.finfo(np.float32).eps


def make(case, precision="fp64", **kw):
    g, meta, system, ew = load(case)
    p = meta["params"]
    fp = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"],
                     precision=precision, h=p["h"], epsc=p["epsc"],
                     omegac=meta["omegac"] or 1.2, **kw)
    return g, meta, system, ew, fp


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_frames_match_reference_playback(precision, tmp_path):
    g, meta, system, ew, fp = make("tip4p216", precision)
    h = meta["params"]["h"]
    R = g["r"]
    heavy = system.mass != 0
    # playback frame k is the state after step k: dump k+1 holds frame k's
    # positions (frames 0-2), frame 3 follows one more step
    fp.md_set_state(R[2], R[2] - R[1])
    base = str(tmp_path / "sim")
    with Playback(base, fp, velocities=True) as pb:
        for _ in range(2):
            fp.md_steps(1)
            pb.write()
    L, r, centred = read_playback(base + ".plb")
    Lv, v, _ = read_playback(base + ".vlb")
    assert not centred and r.shape == (2, system.ns, 3)
    assert np.array_equal(L, g["plb_L"][2:]) and np.array_equal(Lv, g["vlb_L"][2:])
    # positions to one float rounding (FP64 states agree with cook to 1e-9)
    ptol = 2 * F32 * 32 if precision == "fp64" else 2e-6 + 2 * F32 * 32
    assert np.abs(r - g["plb_r"][2:]).max() <= ptol
    # velocities r1/h of the massive sites; a massless site's r1 is not moved
    # by the step (cook's vlb repeats the dependant velocity of the start)
    vtol = 2 * F32 * 128 if precision == "fp64" else 2e-6 / h
    assert np.abs(v[:, heavy] - g["vlb_r"][2:, heavy]).max() <= vtol
    assert np.array_equal(v[0, ~heavy], v[1, ~heavy])
    assert np.allclose(v[0, ~heavy], ((R[2] - R[1]) / h)[~heavy], rtol=0, atol=1e-4)


@pytest.mark.parametrize("flags", [2, 4, 6])
def test_shifted_and_centred_frames(flags):
    g, meta, system, ew, fp = make("spce216")
    R = g["r"]
    fp.md_set_state(R[2], R[2] - R[1])
    fp.md_steps(2)
    r, r1 = fp.md_get_state()
    L, fr = fp.playback_frame("plb", flags)
    d = r.copy()
    if flags & 2:
        d = d - 0.5 * r1
    if flags & 4:
        d = d - 0.5 * np.asarray(ew["L"])
    assert np.array_equal(fr, d.astype(np.float32))
    _, vf = fp.playback_frame("vlb")
    assert np.array_equal(vf, ((1.0 / meta["params"]["h"]) * r1).astype(np.float32))


def test_drude_playback_frame():
    g, meta, system, ew = load("drude216")
    p = meta["params"]
    fp = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"],
                     precision="fp64", h=p["h"], epsc=p["epsc"], omegac=meta["omegac"])
    ns = system.ns
    R, RD = g["r"], g["rD"]
    fp.md_set_state(np.vstack([R[4], RD[4]]), np.vstack([R[4] - R[3], RD[3]]))
    fp.md_steps(2)
    r, _ = fp.md_get_state()
    _, fr = fp.playback_frame("dlb")
    assert np.array_equal(fr, (r[:ns] + r[ns:]).astype(np.float32))
    # a build without Drude charges has no .dlb
    g2, _, _, _, fp2 = make("spce216")
    fp2.md_set_state(g2["r"][2], g2["r"][2] - g2["r"][1])
    with pytest.raises(M.MGError):
        fp2.playback_frame("dlb")
