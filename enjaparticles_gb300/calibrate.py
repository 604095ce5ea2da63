"""Batched differentiable calibration: recover each scene's viscosity from
its trajectory.

For every scene s of a batch the loss is the mean, over the checkpoint times
t = K, 2K, ..., T of the recorded rollout, of (1/N_s) sum_i rho(|x_i,t - x*_i,t|),
x* the trajectory of the scene run with its hidden viscosity and rho the Huber
function with delta = 0.01 h (quadratic below delta, linear above).  Why not
the plain squared distance of the final positions: in some scenes a few
particles change their wall contact by a step when the viscosity changes and
end up a fraction of h away from their targets; with a squared loss they
dominate it, making it flat over much of the viscosity range with minima
away from the true value.  Positions at earlier times and a loss whose
gradient per particle is bounded leave the smooth response of all the other
particles in charge.  Each iteration runs, for all scenes at once:
    rewind -> record (T steps, checkpoint every K) -> trajectory loss -> backward
and takes one gradient step per scene on log(mu_s) (iRprop-: sign-based steps
that adapt per scene).  Device buffers are torch tensors; the work is done by
the library's batched kernels.
"""
import math

import numpy as np


def rprop_step(theta, grad, state, step0=0.1, grow=1.2, shrink=0.5, step_min=1e-7, step_max=0.5):
    """One iRprop- update of the parameter vector theta (numpy, in place).

    Each component moves against the sign of its gradient by its own step,
    which grows while the sign holds and halves when it flips (and that
    component then skips one move).  The steps do not depend on the
    gradients' magnitudes, which differ by orders of magnitude between scenes
    and shrink by orders of magnitude near the optimum."""
    prev = state.setdefault("prev", np.zeros_like(theta))
    step = state.setdefault("step", np.full_like(theta, step0))
    sign = np.sign(grad) * np.sign(prev)
    step[sign > 0] = np.minimum(step[sign > 0] * grow, step_max)
    step[sign < 0] = np.maximum(step[sign < 0] * shrink, step_min)
    g = np.where(sign < 0, 0.0, grad)
    theta -= np.sign(g) * step
    prev[:] = g
    return theta


def checkpoints(nsteps, K):
    """Number of checkpoint times (0, K, 2K, ..., nsteps) of a recorded rollout."""
    K = min(K, nsteps)
    return (nsteps + K - 1) // K + 1


def record_targets(batch, viscosities, nsteps, K, dt, torch):
    """Run every scene with its viscosity from the batch's current state and
    return its trajectory at the checkpoint times (device tensor)."""
    for s, mu in enumerate(viscosities):
        batch.set_viscosity(s, float(np.float32(mu)))
    batch.adjoint_record(dt, nsteps, K)
    traj = torch.zeros((checkpoints(nsteps, K), batch.nslots, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    batch.trajectory(traj.data_ptr())
    batch.adjoint_rewind()
    return traj


def calibrate_viscosity(batch, targets, mu0, iterations=50, nsteps=100, K=10, dt=0.001, step0=0.1, huber=0.01,
                        mu_bounds=(1e-4, 0.5), on_iteration=None):
    """Gradient descent on every scene's viscosity at once.

    batch    an enjaparticles_gb300.batch.Batch holding the initial states
    targets  device tensor (checkpoints(nsteps, K), nslots, 4): the target
             trajectories (record_targets)
    mu0      initial viscosities (one per scene)
    Returns (mu, history) with history[k] = (losses, mus) before step k.
    """
    import torch
    S = batch.nscenes
    grads = torch.zeros_like(targets)
    theta = np.log(np.asarray(mu0, np.float64))
    state = {}
    lo, hi = math.log(mu_bounds[0]), math.log(mu_bounds[1])
    history = []
    for k in range(iterations):
        mus = np.exp(theta)
        for s in range(S):
            batch.set_viscosity(s, float(np.float32(mus[s])))
        if k > 0:
            batch.adjoint_rewind()
        batch.adjoint_record(dt, nsteps, K)
        torch.cuda.synchronize()
        losses = batch.loss_traj(targets.data_ptr(), grads.data_ptr(), huber)
        dmu = np.asarray(batch.adjoint_backward_traj(grads.data_ptr()), np.float64)
        history.append((np.asarray(losses), mus.copy()))
        if on_iteration:
            on_iteration(k, losses, mus, dmu)
        theta = rprop_step(theta, dmu * mus, state, step0=step0)  # dL/dlog(mu) = mu dL/dmu
        np.clip(theta, lo, hi, out=theta)
    batch.adjoint_rewind()
    return np.exp(theta), history
