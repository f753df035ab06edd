"""Helpers of the adjoint checks (test harness only): per-type parameters of
a system, the chain rule from type-pair to type gradients, central
differences of the oracle, and a torch.autograd.Function around the GPU
adjoint."""
import copy

import numpy as np

C6 = 2.0 ** (1.0 / 6.0)


def type_params(system):
    """(eps [K] > 0, sigma [A]) of every type (cook's EvdW = -eps, RvdW = sigma 2^(1/6)/2)"""
    return -np.asarray(system.typeE, float), 2 * np.asarray(system.typeR, float) / C6


def with_params(system, eps=None, sig=None, q=None):
    s = copy.copy(system)
    e0, s0 = type_params(system)
    if eps is not None:
        s.typeE = -np.asarray(eps, float)
    if sig is not None:
        s.typeR = np.asarray(sig, float) * C6 / 2
    if q is not None:
        s.q = np.asarray(q, float)
    return s


def pair_to_type(dP, system):
    """[nt,nt,2] type-pair gradients (a<=b) -> ([nt] d/d eps_t, [nt] d/d sigma_t)
    through eps_ab = sqrt(eps_a eps_b), sigma_ab = (sigma_a + sigma_b)/2"""
    eps, _ = type_params(system)
    nt = len(eps)
    de, ds = np.zeros(nt), np.zeros(nt)
    for a in range(nt):
        for b in range(a, nt):
            ge, gs = dP[a, b]
            if ge == 0 and gs == 0:
                continue
            eab = np.sqrt(eps[a] * eps[b])
            if a == b:
                de[a] += ge
                ds[a] += gs
            else:
                if eps[a] > 0:
                    de[a] += ge * eab / (2 * eps[a])
                if eps[b] > 0:
                    de[b] += ge * eab / (2 * eps[b])
                ds[a] += 0.5 * gs
                ds[b] += 0.5 * gs
    return de, ds


def observables(orc_factory, system, r, target=None):
    """E, W (LJ sum r.f + E_el) and the loss mean |F - target|^2 of the oracle"""
    o = orc_factory(system)
    f, en = o.forces(r, measure=True, nthreads=8)
    E = en["el"] + en["lj"]
    W = en["vir"] + en["el"]
    loss = None if target is None else float(((f - target) ** 2).mean())
    return E, W, loss, f


# ------------------------------------------------- torch.autograd wrapper --

def charge_groups_grad(dq, system, q_groups):
    """the gradient of charge parameters from per-site dX/dq_i: parameter k
    sets q = w * theta_k on the sites of every (type, w) of q_groups[k], so
    dX/dtheta_k = sum over those (type, w) of w * sum of dX/dq_i"""
    return np.array([sum(w * dq[system.type == t].sum() for t, w in grp) for grp in q_groups])


def make_force_match(M, frames, targets, system, ew, lj_types, q_types):
    """A torch.autograd.Function of theta = (eps_t, sigma_t for t in lj_types,
    then one charge parameter per entry of q_types) -> force-matching loss
    mean |F(theta) - target|^2 over the frames, with the gradient from the GPU
    adjoint (mg_adjoint).  An entry of q_types is a type (every site of it
    takes the parameter as its charge) or a list of (type, weight): the sites
    of each type take weight * parameter, which keeps a neutral molecule or
    an ion pair neutral (e.g. [(H, 1), (O, -2)])."""
    import torch

    groups = [[(t, 1.0)] if np.isscalar(t) else list(t) for t in q_types]

    def unpack(theta):
        th = theta.detach().cpu().numpy().astype(np.float64)
        eps, sig = type_params(system)
        eps, sig, q = eps.copy(), sig.copy(), system.q.copy()
        n = len(lj_types)
        for k, t in enumerate(lj_types):
            eps[t], sig[t] = th[k], th[n + k]
        for k, grp in enumerate(groups):
            for t, w in grp:
                q[system.type == t] = w * th[2 * n + k]
        return with_params(system, eps=eps, sig=sig, q=q)

    class ForceMatch(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta):
            s = unpack(theta)
            fp = M.ForcePath(s, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"], precision="fp64")
            loss, grad = 0.0, np.zeros(theta.numel())
            n = len(lj_types)
            nf = sum(t.size for t in targets)
            for r, tgt in zip(frames, targets):
                f, _ = fp.forces(r)
                d = f - tgt
                loss += float((d ** 2).sum()) / nf
                adj = fp.adjoint(r, 2 * d / nf)
                de, ds = pair_to_type(adj["dLp"], s)
                for k, t in enumerate(lj_types):
                    grad[k] += de[t]
                    grad[n + k] += ds[t]
                if groups:
                    grad[2 * n:] += charge_groups_grad(adj["dLq"], s, groups)
            fp.close()
            ctx.save_for_backward(torch.tensor(grad, dtype=theta.dtype))
            return theta.new_tensor(loss)

        @staticmethod
        def backward(ctx, gout):
            (grad,) = ctx.saved_tensors
            return gout * grad

    return ForceMatch, unpack
