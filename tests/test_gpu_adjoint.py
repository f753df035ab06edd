"""The GPU adjoint (mg_adjoint, FP64) against the oracle's analytic gradient
and against central differences (h = 1e-5 relative) of the GPU path itself;
a force-matching fit through a torch.autograd.Function built on it."""
import numpy as np
import pytest

import macsimus_gb300 as M
from adjoint_harness import make_force_match, pair_to_type, type_params, with_params
from golden_cases import load
from macsimus_gb300 import forcefield as ff
from oracle import oracle as O

pytestmark = pytest.mark.gpu

LJ = [ff.TYPE_ORDER.index(n) for n in ("O", "NA", "CL")]


def gpu(system, ew):
    return M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"], precision="fp64")


def observe(system, ew, r, target):
    fp = gpu(system, ew)
    f, en = fp.forces(r, measure=True)
    return en["el"] + en["lj"], en["vir"] + en["el"], float(((f - target) ** 2).mean())


def test_adjoint_matches_oracle():
    g, meta, system, ew = load("brine532")
    r = g["r"][1]
    fp = gpu(system, ew)
    f, _ = fp.forces(r)
    rng = np.random.default_rng(2)
    gl = rng.normal(size=f.shape) * 1e-3
    a = fp.adjoint(r, gl)
    o = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"]).adjoint(r, gl)
    assert abs(a["E"] - o["E"]) < 1e-10 * abs(o["E"])
    assert abs(a["W"] - o["W"]) < 1e-10 * abs(o["W"])
    for k in ("dEp", "dWp", "dLp"):
        scale = np.abs(o[k]).max()
        assert np.abs(a[k] - o[k]).max() < 1e-10 * scale, k
    for k in ("dEq", "dLq"):
        assert np.abs(a[k] - o[k]).max() < 1e-9 * np.abs(o[k]).max(), k


def test_adjoint_matches_gpu_central_differences():
    g, meta, system, ew = load("brine532")
    r = g["r"][0]
    fp = gpu(system, ew)
    f0, _ = fp.forces(r)
    target = f0 * 1.01 + 5.0
    a = fp.adjoint(r, 2 * (f0 - target) / f0.size)
    gE, gW, gL = (pair_to_type(a[k], system) for k in ("dEp", "dWp", "dLp"))
    eps, sig = type_params(system)
    for t in LJ:
        for k, (p, name) in enumerate(((eps, "eps"), (sig, "sig"))):
            h = 1e-5 * p[t]
            pp, pm = p.copy(), p.copy()
            pp[t] += h
            pm[t] -= h
            vp = observe(with_params(system, **{name: pp}), ew, r, target)
            vm = observe(with_params(system, **{name: pm}), ew, r, target)
            for idx, grad in enumerate((gE, gW, gL)):
                fd = (vp[idx] - vm[idx]) / (2 * h)
                assert abs(grad[k][t] - fd) <= 1e-5 * abs(fd) + 1e-7 * abs(vp[idx]) / p[t], \
                    (t, name, idx, grad[k][t], fd)
    # a neutral change of the water charges: q_H + d, q_O - 2 d
    iH, iO = ff.TYPE_ORDER.index("H"), ff.TYPE_ORDER.index("O")
    d = 1e-5 * ff.ELECTRON
    an = {k: a[k][system.type == iH].sum() - 2 * a[k][system.type == iO].sum()
          for k in ("dEq", "dLq")}
    qp, qm = system.q.copy(), system.q.copy()
    for q, sgn in ((qp, 1), (qm, -1)):
        q[system.type == iH] += sgn * d
        q[system.type == iO] -= 2 * sgn * d
    vp = observe(with_params(system, q=qp), ew, r, target)
    vm = observe(with_params(system, q=qm), ew, r, target)
    assert abs(an["dEq"] - (vp[0] - vm[0]) / (2 * d)) < 1e-6 * abs(an["dEq"])
    assert abs(an["dEq"] - (vp[1] - vm[1]) / (2 * d)) < 1e-6 * abs(an["dEq"])
    assert abs(an["dLq"] - (vp[2] - vm[2]) / (2 * d)) < 1e-5 * abs(an["dLq"])


def test_force_matching_fit_recovers_perturbed_parameters():
    """targets: forces of the same frames with sigma +3 % and epsilon -5 %
    for every LJ type; 200 Adam steps (cosine-decayed step) on the relative
    parameter changes.  The forces are dominated by the LJ repulsion
    eps sigma^12, so the fit lands on the valley (1+de)(1+ds)^12 = const
    quickly and moves along it slowly: the check is the loss and that
    combination, not eps and sigma one by one."""
    torch = pytest.importorskip("torch")
    g, meta, system, ew = load("brine532")
    frames = [g["r"][k] for k in range(g["r"].shape[0])]
    eps, sig = type_params(system)
    pert = with_params(system, eps=np.where(np.isin(np.arange(len(eps)), LJ), eps * 0.95, eps),
                       sig=np.where(np.isin(np.arange(len(sig)), LJ), sig * 1.03, sig))
    fpt = gpu(pert, ew)
    targets = [fpt.forces(r)[0] for r in frames]
    ForceMatch, unpack = make_force_match(M, frames, targets, system, ew, LJ, [])
    theta0 = np.concatenate([eps[LJ], sig[LJ]])
    x = torch.zeros(len(theta0), dtype=torch.float64, requires_grad=True)  # relative change
    t0 = torch.tensor(theta0)
    opt = torch.optim.Adam([x], lr=1e-2)
    sched = torch.optim.lr_scheduler.CosineAnnealingLR(opt, 200)
    first = None
    for _ in range(200):
        opt.zero_grad()
        loss = ForceMatch.apply(t0 * (1 + x))
        loss.backward()
        opt.step()
        sched.step()
        first = first if first is not None else float(loss)
    last = float(loss)
    assert last < 1e-3 * first
    fitted = x.detach().numpy()
    rep = (1 + fitted[:3]) * (1 + fitted[3:]) ** 12 / (0.95 * 1.03 ** 12) - 1
    # O (1000 sites) is well determined; the 16 + 16 ions less so
    assert abs(rep[0]) < 0.02 and np.all(np.abs(rep) < 0.05), rep
    assert np.all(np.abs(fitted[3:] - 0.03) < 0.01), fitted
