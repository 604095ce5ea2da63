"""Batched differentiable calibration: recover each scene's viscosity from
its final positions.

For every scene s of a batch the loss is L_s(mu_s) = (1/N_s) sum |x_T - x*_T|^2,
x* the final positions of the scene run with its hidden viscosity.  Each
iteration runs, for all scenes at once:
    rewind -> record (nsteps steps, checkpoint every K) -> loss -> backward
and takes one gradient step per scene on log(mu_s) (Adam: its steps do not
depend on each scene's loss scale, which differs by orders of magnitude
between scenes).  Device buffers are torch tensors; the work is done by the
library's batched kernels.
"""
import math

import numpy as np


def adam_steps(theta, grad, state, lr, b1=0.9, b2=0.999, eps=1e-12):
    """One Adam update of the parameter vector theta (numpy, in place)."""
    state["t"] += 1
    m = state.setdefault("m", np.zeros_like(theta))
    v = state.setdefault("v", np.zeros_like(theta))
    m[:] = b1 * m + (1 - b1) * grad
    v[:] = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1 ** state["t"])
    vh = v / (1 - b2 ** state["t"])
    theta -= lr * mh / (np.sqrt(vh) + eps)
    return theta


def calibrate_viscosity(batch, target_ptr, mu0, iterations=50, nsteps=100, K=10, dt=0.001, lr=0.15, lr_end=0.01,
                        mu_bounds=(1e-4, 0.5), torch=None, on_iteration=None):
    """Gradient descent on every scene's viscosity at once.

    batch       an enjaparticles_gb300.batch.Batch holding the initial states
    target_ptr  device address of the target final positions (slot layout)
    mu0         initial viscosities (one per scene)
    Returns (mu, history) with history[k] = (losses, mus) before step k.
    """
    import torch as _torch
    torch = torch or _torch
    S = batch.nscenes
    grad = torch.zeros((batch.nslots, 4), dtype=torch.float32, device="cuda")
    theta = np.log(np.asarray(mu0, np.float64))
    state = {"t": 0}
    lo, hi = math.log(mu_bounds[0]), math.log(mu_bounds[1])
    history = []
    first = True
    for k in range(iterations):
        mus = np.exp(theta)
        for s in range(S):
            batch.set_viscosity(s, float(np.float32(mus[s])))
        if not first:
            batch.adjoint_rewind()
        batch.adjoint_record(dt, nsteps, K)
        first = False
        torch.cuda.synchronize()
        losses = batch.loss_mse(target_ptr, grad.data_ptr())
        dmu = np.asarray(batch.adjoint_backward(dpos=grad.data_ptr()), np.float64)
        history.append((np.asarray(losses), mus.copy()))
        if on_iteration:
            on_iteration(k, losses, mus, dmu)
        lr_k = lr_end + 0.5 * (lr - lr_end) * (1 + math.cos(math.pi * k / max(iterations - 1, 1)))
        theta = adam_steps(theta, dmu * mus, state, lr_k)  # dL/dlog(mu) = mu dL/dmu
        np.clip(theta, lo, hi, out=theta)
    batch.adjoint_rewind()
    return np.exp(theta), history
