"""Test-side wrapper of the differentiable rollout and its finite-difference
check.

SPHRollout is a torch.autograd.Function whose forward is a recorded rollout
(sph_adjoint_record) and whose backward is the library's adjoint
(sph_adjoint_backward).  It lives here, in the tests, as the harness that
checks the C ABI; the library itself has no torch dependency.

fd_gradient is the checker: central differences of a loss of the final
positions, each loss evaluated by the FP64 rollout of the oracle.  Stencils
whose two sides took different wall / friction / clamp branches anywhere in
the rollout are rejected (their difference quotient measures a jump, not a
derivative).
"""
import ctypes as C

import numpy as np
import torch

import oracle_bind as ob


class SPHRollout(torch.autograd.Function):
    """pos_T = rollout(pos0, vel0, veleval0; viscosity), differentiable in all four."""

    @staticmethod
    def forward(ctx, pos0, vel0, veleval0, visc, system, dt, nsteps, K):
        sp = system.params()[0]
        sp.viscosity = float(visc.item())
        system.updateParams(sp)
        system.upload(pos0.detach().cpu().numpy(), vel0.detach().cpu().numpy(),
                      veleval0.detach().cpu().numpy())
        system.adjoint_record(dt, nsteps, K)
        n = pos0.shape[0]
        ctx.system = system
        ctx.n = n
        ctx.dev = pos0.device
        return torch.from_numpy(system.get("pos_u", n).copy()).to(pos0.device)

    @staticmethod
    def backward(ctx, g):
        g = g.detach().to(ctx.dev, torch.float32).contiguous()
        n = ctx.n
        dp = torch.zeros((n, 4), dtype=torch.float32, device=ctx.dev)
        dv = torch.zeros_like(dp)
        de = torch.zeros_like(dp)
        # the library runs on its own stream: torch's writes must be done
        torch.cuda.synchronize(ctx.dev)
        dmu = ctx.system.adjoint_backward(dpos=g.data_ptr(), out_pos=dp.data_ptr(), out_vel=dv.data_ptr(),
                                          out_veleval=de.data_ptr())
        torch.cuda.synchronize(ctx.dev)
        return dp, dv, de, torch.tensor(dmu, dtype=torch.float64), None, None, None, None


def loss64(pos_T, target=None, weights=None):
    """FP64 loss of final positions: mean squared distance to `target`, or
    sum(weights * pos) when weights are given."""
    p = np.asarray(pos_T, np.float64)[:, :3]
    if weights is not None:
        return float(np.sum(weights * p))
    d = p - np.asarray(target, np.float64)[:, :3]
    return float(np.mean(np.sum(d * d, axis=1)))


def fd_gradient(sp, gs, pos, vel, veleval, dt, nsteps, which, index, eps, target=None, weights=None,
                viscosity=None):
    """Central difference of the FP64 loss along one input coordinate.

    which: "pos", "vel", "veleval" (index = (particle, axis)) or "visc".
    Returns (derivative, branches_agree, neighbours_agree).
    """
    mu0 = float(sp.viscosity) if viscosity is None else float(viscosity)
    base = {"pos": np.asarray(pos, np.float64)[:, :3].copy(), "vel": np.asarray(vel, np.float64)[:, :3].copy(),
            "veleval": (np.zeros_like(np.asarray(pos, np.float64)[:, :3]) if veleval is None
                        else np.asarray(veleval, np.float64)[:, :3].copy())}
    out = []
    for sgn in (1.0, -1.0):
        arrs = {k: v.copy() for k, v in base.items()}
        mu = mu0
        if which == "visc":
            mu = mu0 + sgn * eps
        else:
            arrs[which][index[0], index[1]] += sgn * eps
        pT, _, sb, sn = ob.rollout64(sp, gs, arrs["pos"], arrs["vel"], dt, nsteps, viscosity=mu,
                                     veleval=arrs["veleval"])
        out.append((loss64(pT, target, weights), sb, sn))
    (lp, sbp, snp), (lm, sbm, snm) = out
    return (lp - lm) / (2.0 * eps), sbp == sbm, snp == snm


def rel_err(a, b):
    return abs(a - b) / max(abs(b), 1e-300)
