"""Batches of independent ionic-fluid boxes: the graph-captured batch MD and
the one-launch batch Widom give what the same boxes give one by one."""
import numpy as np
import pytest

import macsimus_gb300 as M
from macsimus_gb300 import configs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def boxes(n=5, seed=11):
    return configs.ionic_boxes(n, seed=seed, nmin=300, nmax=1200)


def args(b):
    return dict(system=b["system"], L=b["L"], cutoff=b["cutoff"], alpha=b["alpha"],
                kappa=b["kappa"], h=b["h"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_md_equals_single_boxes(precision):
    bs = boxes()
    batch = M.Batch([args(b) for b in bs], precision=precision, lanes=3)
    for i, b in enumerate(bs):
        batch.box[i].md_set_state(b["r"], b["r1"])
    en = batch.md_steps(6)
    assert batch.launches > 0
    for i, b in enumerate(bs):
        a = args(b)
        fp = M.ForcePath(a.pop("system"), a.pop("L"), a.pop("cutoff"), a.pop("alpha"),
                         a.pop("kappa"), precision=precision, **a)
        fp.md_set_state(b["r"], b["r1"])
        e1 = fp.md_steps(6)
        rb, r1b = batch.box[i].md_get_state()
        rs, r1s = fp.md_get_state()
        assert np.array_equal(rb, rs) and np.array_equal(r1b, r1s)
        for k in ("el", "lj", "ekin"):
            assert en[i][k] == e1[k]
    # a second call replays the captured graphs
    batch.md_steps(2, measure=False)
    batch.close()


@pytest.mark.parametrize("engine", [1, 0])
def test_fused_batch_md_equals_single_boxes(engine):
    """boxes on the FP32 path with the Ewald passes on the FP32 cores (1) or
    the tensor cores (0): one launch per kernel over all boxes (blockIdx.y =
    box); every box gets the positions, velocities and energies it gets
    alone, bit for bit, and the launches per step do not grow with the
    number of boxes"""
    launches = {}
    for n in (3, 7):
        bs = boxes(n, seed=13)
        batch = M.Batch([dict(args(b), kspace_engine=engine) for b in bs], precision="mixed",
                        lanes=3)
        for i, b in enumerate(bs):
            batch.box[i].md_set_state(b["r"], b["r1"])
        en = batch.md_steps(6)
        assert batch.fused
        batch.md_steps(2, measure=False)
        launches[n] = batch.launches
        for i, b in enumerate(bs):
            a = dict(args(b), kspace_engine=engine)
            fp = M.ForcePath(a.pop("system"), a.pop("L"), a.pop("cutoff"), a.pop("alpha"),
                             a.pop("kappa"), precision="mixed", **a)
            fp.md_set_state(b["r"], b["r1"])
            e1 = fp.md_steps(6)
            fp.md_steps(2, measure=False)
            rb, r1b = batch.box[i].md_get_state()
            rs, r1s = fp.md_get_state()
            assert np.array_equal(rb, rs) and np.array_equal(r1b, r1s)
            for k in ("el", "lj", "ekin", "virc"):
                assert en[i][k] == e1[k], k
            assert en[i]["Ptens"] == e1["Ptens"]
        # Widom into the configurations the batched step left
        w = batch.widom([2], n=20000, seed=3, T=298.0)
        assert all(np.isfinite(x["mu"]) for x in w)
        batch.close()
    assert launches[3] == launches[7]


def test_batch_forces_match_oracle():
    bs = boxes(3, seed=5)
    batch = M.Batch([args(b) for b in bs], precision="fp64")
    for i, b in enumerate(bs):
        f, _ = batch.box[i].forces(b["r"])
        orc = O.Oracle(b["system"], [b["L"]] * 3, b["cutoff"], b["alpha"], b["kappa"])
        fo, _ = orc.forces(b["r"], nthreads=4)
        assert np.sqrt(((f - fo) ** 2).sum() / (fo ** 2).sum()) < 1e-10
    batch.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_widom_equals_single_boxes(precision):
    bs = boxes(4, seed=7)
    batch = M.Batch([args(b) for b in bs], precision=precision)
    for i, b in enumerate(bs):
        batch.box[i].forces(b["r"])
    res = batch.widom([2], n=30000, seed=99, T=298.0)
    for i, b in enumerate(bs):
        one = batch.box[i].widom([2], n=30000, seed=(99 + 0x632BE59BD9B4E019 * i) % 2 ** 64,
                                 T=298.0)
        assert res[i]["sum"] == one["sum"]
        assert res[i]["corr"] == one["corr"]
        orc = O.Oracle(b["system"], [b["L"]] * 3, b["cutoff"], b["alpha"], b["kappa"])
        s, corr, _ = orc.widom(b["r"], [2], [0.0], [0, 0, 0], 30000,
                               (99 + 0x632BE59BD9B4E019 * i) % 2 ** 64, 298.0)
        assert abs(res[i]["sum"] - s) <= (1e-11 if precision == "fp64" else 2e-6) * s
    batch.close()


def test_batch_requires_state():
    bs = boxes(2)
    batch = M.Batch([args(b) for b in bs])
    batch.box[0].md_set_state(bs[0]["r"], bs[0]["r1"])
    with pytest.raises(M.MGError):
        batch.md_steps(1)
    batch.close()


def test_batch_profile_stages():
    """mg_batch_profile: the fused step stage by stage; every stage runs
    (its time is positive) and the steps it takes are ordinary MD steps"""
    bs = boxes(4, seed=17)
    batch = M.Batch([dict(args(b), kspace_engine=0) for b in bs], precision="mixed", lanes=2)
    for i, b in enumerate(bs):
        batch.box[i].md_set_state(b["r"], b["r1"])
    batch.md_steps(2, measure=False)
    assert batch.fused
    st = batch.profile(3)
    assert set(st) == set(M.Batch.PROFILE_STAGES)
    for k in ("cell_list", "pair", "ewald_sk", "ewald_sk_reduce", "ewald_kforce", "shake"):
        assert st[k] > 0, k
    # the profiled steps advanced the boxes like md_steps: the same state as
    # 2 + 3 plain steps from the start
    ref = M.Batch([dict(args(b), kspace_engine=0) for b in bs], precision="mixed", lanes=2)
    for i, b in enumerate(bs):
        ref.box[i].md_set_state(b["r"], b["r1"])
    ref.md_steps(5, measure=False)
    for i in range(len(bs)):
        assert np.array_equal(batch.box[i].md_get_state()[0], ref.box[i].md_get_state()[0])
    batch.close()
    ref.close()
