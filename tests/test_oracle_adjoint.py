"""The oracle's analytic gradients (the adjoint restatement) against central
differences of the oracle's own energies, virial and forces, on the brine
fixture: LJ (eps, sigma) per type and site charges."""
import numpy as np

from adjoint_harness import observables, pair_to_type, type_params, with_params
from golden_cases import load
from macsimus_gb300 import forcefield as ff
from oracle import oracle as O


def setup():
    g, meta, system, ew = load("brine532")
    r = g["r"][0]

    def factory(s):
        return O.Oracle(s, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    return r, system, factory


def test_lj_gradients_match_central_differences():
    r, system, factory = setup()
    rng = np.random.default_rng(0)
    E0, W0, _, F0 = observables(factory, system, r)
    target = F0 + rng.normal(size=F0.shape) * np.abs(F0).mean()
    g = 2 * (F0 - target) / F0.size
    adj = factory(system).adjoint(r, g)
    assert abs(adj["E"] - E0) < 1e-9 * abs(E0)
    assert abs(adj["W"] - W0) < 1e-9 * abs(W0)
    gE = pair_to_type(adj["dEp"], system)
    gW = pair_to_type(adj["dWp"], system)
    gL = pair_to_type(adj["dLp"], system)
    eps, sig = type_params(system)
    for t in [ff.TYPE_ORDER.index(n) for n in ("O", "NA", "CL")]:
        for k, (p, base) in enumerate(((eps, "eps"), (sig, "sig"))):
            h = 1e-5 * p[t]
            vals = []
            for sgn in (1, -1):
                pp = p.copy()
                pp[t] += sgn * h
                s2 = with_params(system, **{base: pp})
                vals.append(observables(factory, s2, r, target))
            for idx, grad in ((0, gE), (1, gW), (2, gL)):
                fd = (vals[0][idx] - vals[1][idx]) / (2 * h)
                an = grad[k][t]
                assert abs(an - fd) <= 2e-6 * max(abs(fd), 1e-3 * abs(vals[0][idx]) / p[t]), \
                    (t, base, idx, an, fd)


def test_charge_gradients_match_central_differences():
    r, system, factory = setup()
    rng = np.random.default_rng(1)
    E0, W0, _, F0 = observables(factory, system, r)
    target = F0 + rng.normal(size=F0.shape) * np.abs(F0).mean()
    g = 2 * (F0 - target) / F0.size
    adj = factory(system).adjoint(r, g)
    for i in (0, 1, 1500, 1520):
        h = 1e-5 * ff.ELECTRON
        vals = []
        for sgn in (1, -1):
            q = system.q.copy()
            q[i] += sgn * h
            vals.append(observables(factory, with_params(system, q=q), r, target))
        fdE = (vals[0][0] - vals[1][0]) / (2 * h)
        fdW = (vals[0][1] - vals[1][1]) / (2 * h)
        fdL = (vals[0][2] - vals[1][2]) / (2 * h)
        assert abs(adj["dEq"][i] - fdE) < 1e-6 * abs(fdE) + 1e-9, (i, adj["dEq"][i], fdE)
        assert abs(adj["dEq"][i] - fdW) < 1e-6 * abs(fdW) + 1e-9
        assert abs(adj["dLq"][i] - fdL) < 1e-5 * abs(fdL) + 1e-12, (i, adj["dLq"][i], fdL)
