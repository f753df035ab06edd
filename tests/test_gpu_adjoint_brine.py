"""The adjoint at the stated size: 4096 SPC/E + 128 Na+ + 128 Cl- (12544
sites, cutoff 10 A, alpha 0.31/A, |n| <= 12), 64 seeded frames of an MD run.

Parameters: epsilon and sigma of O, Na, Cl and two charges under the
neutrality constraint (q_H with q_O = -2 q_H; q_Na with q_Cl = -q_Na).
Checks on one frame: the GPU gradients of E, W and the force-matching loss
against FP64 central differences (h = 1e-5 relative) of the GPU path and
against the oracle's analytic gradient.  Then 200 Adam steps of a
force-matching fit over the 64 frames to targets made with sigma +3 % and
epsilon -5 % for every type (torch.autograd.Function over the C ABI, test
harness only)."""
import numpy as np
import pytest

import macsimus_gb300 as M
from adjoint_harness import (charge_groups_grad, make_force_match, pair_to_type, type_params,
                             with_params)
from macsimus_gb300 import configs
from macsimus_gb300 import forcefield as ff
from oracle import oracle as O

pytestmark = pytest.mark.gpu

LJ = [ff.TYPE_ORDER.index(n) for n in ("O", "NA", "CL")]
iH, iO, iNA, iCL = (ff.TYPE_ORDER.index(n) for n in ("H", "O", "NA", "CL"))
QG = [[(iH, 1.0), (iO, -2.0)], [(iNA, 1.0), (iCL, -1.0)]]


@pytest.fixture(scope="module")
def brine():
    w = configs.equilibrate(configs.workload("brine4352", seed=11), steps=200)
    ew = dict(L=np.array([w["L"]] * 3), cutoff=w["cutoff"], alpha=w["alpha"], kappa=w["kappa"])
    fp = M.ForcePath(w["system"], ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"],
                     precision="mixed", h=0.002, epsc=1e-7)
    fp.md_set_state(w["r"], w["r1"])
    frames = []
    for _ in range(64):
        fp.md_steps(10, measure=False)
        frames.append(fp.md_get_state()[0].copy())
    fp.close()
    return w["system"], ew, frames


def fp64(system, ew):
    return M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"], precision="fp64")


def qparams(system):
    return np.array([system.q[system.type == iH][0], system.q[system.type == iNA][0]])


def with_theta(system, eps, sig, qp):
    q = system.q.copy()
    for grp, v in zip(QG, qp):
        for t, wt in grp:
            q[system.type == t] = wt * v
    return with_params(system, eps=eps, sig=sig, q=q)


def observe(system, ew, r, target):
    f, en = fp64(system, ew).forces(r, measure=True)
    return en["el"] + en["lj"], en["vir"] + en["el"], float(((f - target) ** 2).mean())


def perturbed(system):
    eps, sig = type_params(system)
    lj = np.isin(np.arange(len(eps)), LJ)
    return with_params(system, eps=np.where(lj, eps * 0.95, eps), sig=np.where(lj, sig * 1.03, sig))


def test_brine_gradients_match_central_differences_and_oracle(brine):
    system, ew, frames = brine
    r = frames[7]
    eps, sig = type_params(system)
    target = fp64(perturbed(system), ew).forces(r)[0]
    fp = fp64(system, ew)
    f0, _ = fp.forces(r)
    g = 2 * (f0 - target) / f0.size
    a = fp.adjoint(r, g)
    # the oracle's analytic gradient (FP64 reference)
    o = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"]).adjoint(r, g)
    for k in ("dEp", "dWp", "dLp"):
        assert np.abs(a[k] - o[k]).max() < 1e-9 * np.abs(o[k]).max(), k
    for k in ("dEq", "dLq"):
        assert np.abs(a[k] - o[k]).max() < 1e-8 * np.abs(o[k]).max(), k
    # central differences, h = 1e-5 relative, of E, W and the loss
    grads = [pair_to_type(a[k], system) for k in ("dEp", "dWp", "dLp")]
    qgrad = [charge_groups_grad(a[k], system, QG) for k in ("dEq", "dEq", "dLq")]
    qp = qparams(system)
    for idx in range(3):
        for t in LJ:
            for kk, (p, name) in enumerate(((eps, "eps"), (sig, "sig"))):
                h = 1e-5 * p[t]
                pp, pm = p.copy(), p.copy()
                pp[t] += h
                pm[t] -= h
                vp = observe(with_params(system, **{name: pp}), ew, r, target)[idx]
                vm = observe(with_params(system, **{name: pm}), ew, r, target)[idx]
                fd = (vp - vm) / (2 * h)
                assert abs(grads[idx][kk][t] - fd) <= 1e-5 * abs(fd) + 1e-7 * abs(vp) / p[t], \
                    (idx, t, name, grads[idx][kk][t], fd)
        for k in range(2):
            h = 1e-5 * abs(qp[k])
            qpp, qpm = qp.copy(), qp.copy()
            qpp[k] += h
            qpm[k] -= h
            vp = observe(with_theta(system, eps, sig, qpp), ew, r, target)[idx]
            vm = observe(with_theta(system, eps, sig, qpm), ew, r, target)[idx]
            fd = (vp - vm) / (2 * h)
            assert abs(qgrad[idx][k] - fd) <= 1e-5 * abs(fd) + 1e-9 * abs(vp) / abs(qp[k]), \
                (idx, k, qgrad[idx][k], fd)


def test_brine_force_matching_fit_64_frames(brine):
    """200 Adam steps over the 64 frames on (eps, sigma) of O, Na, Cl and
    the two neutral charge parameters; the targets change only eps and
    sigma, so the fitted charges stay put and the repulsion eps sigma^12 of
    every type is recovered"""
    torch = pytest.importorskip("torch")
    system, ew, frames = brine
    eps, sig = type_params(system)
    fpt = fp64(perturbed(system), ew)
    targets = [fpt.forces(r)[0] for r in frames]
    fpt.close()
    ForceMatch, unpack = make_force_match(M, frames, targets, system, ew, LJ, QG)
    theta0 = np.concatenate([eps[LJ], sig[LJ], qparams(system)])
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
        first = first if first is not None else float(loss.detach())
    last = float(loss.detach())
    fitted = x.detach().numpy()
    print("brine fit: loss %.3g -> %.3g, relative changes %s" % (first, last, np.round(fitted, 4)))
    assert last < 1e-2 * first
    rep = (1 + fitted[:3]) * (1 + fitted[3:6]) ** 12 / (0.95 * 1.03 ** 12) - 1
    assert abs(rep[0]) < 0.02 and np.all(np.abs(rep) < 0.06), rep
    assert np.all(np.abs(fitted[6:]) < 0.01), fitted
