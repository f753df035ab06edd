"""The playback file layout (sim/simils.c openplayback/writeplayback and
readplayback) on the CPU: cook's own .plb/.vlb of the tip4p216 fixture
re-encoded and read back, and the old fixed-L header."""
import os

import numpy as np

from golden_cases import load
from macsimus_gb300.playback import read_playback


def test_reads_variable_box_layout(tmp_path):
    g, meta, system, ew = load("tip4p216")
    for ext in ("plb", "vlb"):
        fn = str(tmp_path / ("sim." + ext))
        with open(fn, "wb") as f:
            np.array([system.ns, -3], np.float32).tofile(f)
            for L, r in zip(g[ext + "_L"], g[ext + "_r"]):
                L.astype(np.float32).tofile(f)
                r.astype(np.float32).tofile(f)
        # cook's size rule: 8 bytes of header, 12 (ns + 1) per frame
        assert os.path.getsize(fn) == 8 + 12 * (system.ns + 1) * len(g[ext + "_L"])
        L, r, centred = read_playback(fn)
        assert not centred
        assert np.array_equal(L, g[ext + "_L"]) and np.array_equal(r, g[ext + "_r"])


def test_reads_fixed_cube_header(tmp_path):
    fn = str(tmp_path / "old.plb")
    r = np.random.default_rng(1).random((3, 5, 3), dtype=np.float32)
    with open(fn, "wb") as f:
        np.array([5, 12.5], np.float32).tofile(f)
        r.tofile(f)
    L, rr, _ = read_playback(fn)
    assert np.array_equal(rr, r) and np.all(L == 12.5)
