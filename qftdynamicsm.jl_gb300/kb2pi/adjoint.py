"""Differentiable late-time observables of a KB run (kb_adjoint).

The loss is L = sum_k w_n[k] n(k, t_final) + w_E E(t_final) over cubic
orbits k; kb_adjoint returns dL/dlambda, dL/dm^2 and dL/dn_init per orbit from
one forward pass with state copies every ckpt_every steps and one reverse pass.
The reference's Julia side would expose this through a ChainRulesCore rrule
(the Julia glue defines one); in Python the same call sits behind a
torch.autograd.Function.

Helpers build the loss and initial state of the adjoint workload: the average
of n over radial shells of |p| and an occupation made of Gaussian bumps in |p|.
"""
from __future__ import annotations

import numpy as np

from . import capi


def shell_weights(k2, deg, nshells=8):
    """w_n such that sum_k w_n[k] n[k] = sum over shells of the deg-weighted
    mean of n in the shell; shells split [0, max |p|] into nshells equal bins."""
    p = np.sqrt(np.asarray(k2, float))
    deg = np.asarray(deg, float)
    edges = np.linspace(0.0, p.max(), nshells + 1)
    idx = np.clip(np.searchsorted(edges, p, side="right") - 1, 0, nshells - 1)
    w = np.zeros_like(p)
    for s in range(nshells):
        m = idx == s
        if m.any():
            w[m] = deg[m] / deg[m].sum()
    return w


def bump_basis(k2, nbumps=8):
    """B[b, k] = exp(-(|p_k| - c_b)^2 / (2 s^2)), c_b = (b + 1/2) s, s = max|p| / nbumps;
    the occupation is n_init = amplitudes @ B."""
    p = np.sqrt(np.asarray(k2, float))
    s = p.max() / nbumps
    c = (np.arange(nbumps) + 0.5) * s
    return np.exp(-((p[None, :] - c[:, None]) ** 2) / (2 * s * s))


def params_for(cfg, flags):
    return capi.KbParams(Ns=cfg["Ns"], sdim=3, M=cfg["M"], N=cfg.get("N", 4), pexp=cfg.get("pexp", 1),
                         precision=capi.KB_PREC_FP64, device=cfg.get("device", 0), flags=flags, dt=cfg["dt"],
                         lam=cfg["lam"], mass2=cfg.get("mass2", 1.0), mass=cfg.get("mass", 1.0))


def loss_and_grad(cfg, n_init, t_final, w_n=None, w_E=0.0, ckpt_every=20, init_mass=None):
    """One kb_adjoint call on a fresh FP64 handle; returns the dict of Handle.adjoint.
    The memory integrals run split in two (memint_split 1): twice the CTAs for the
    few orbit chunks of the small lattices gradients are taken on (results differ
    from the whole-chunk kernel in rounding only)."""
    h = capi.Handle([params_for(cfg, ckpt_every)])
    try:
        h.set_tuning(memint_split=1)
        mi = cfg.get("mass", 1.0) if init_mass is None else init_mass
        return h.adjoint(n_init, mi, t_final, w_n=w_n, w_E=w_E, ckpt_every=ckpt_every)
    finally:
        h.close()


def make_function():
    """torch.autograd.Function computing L(lambda, m^2, amplitudes) with the
    adjoint as its backward; imported lazily so that the module has no hard
    torch dependency."""
    import torch

    class KBLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, lam, mass2, amps, cfg, basis, t_final, w_n, w_E, ckpt_every):
            c = dict(cfg, lam=float(lam), mass2=float(mass2))
            n0 = amps.detach().cpu().double().numpy() @ basis
            r = loss_and_grad(c, n0, t_final, w_n=w_n, w_E=w_E, ckpt_every=ckpt_every)
            ctx.grads = (torch.tensor(r["lambda"], dtype=torch.float64),
                         torch.tensor(r["mass2"], dtype=torch.float64),
                         torch.from_numpy(basis @ r["n_init"]))
            return torch.tensor(r["loss"], dtype=torch.float64)

        @staticmethod
        def backward(ctx, g):
            gl, gm, ga = ctx.grads
            return g * gl, g * gm, g * ga, None, None, None, None, None, None

    return KBLoss
