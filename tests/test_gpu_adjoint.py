"""Differentiable rollout: the library's adjoint (through a torch.autograd.Function
used only here) against FP64 central finite differences of the oracle's
double-state rollout.

Stencils whose +eps and -eps rollouts took different wall / friction / clamp
branches are rejected and the coordinate is resampled: across such a jump the
difference quotient is not a derivative.
"""
import numpy as np
import pytest
import torch

from adjoint_harness import SPHRollout, fd_gradient, loss64, rel_err
from enjaparticles_gb300 import abi
from enjaparticles_gb300.scenes import dambreak, normal, rollout_case, sample_coordinates, uniform
from enjaparticles_gb300.sph import SPH

pytestmark = pytest.mark.gpu

DT = 0.001


def _system(n, viscosity=0.01, exact=False):
    sp, g, gs = abi.dambreak_params(n, viscosity)
    return SPH(sp, g, n, gs, exact=exact), sp, g, gs


def _grads(system, pos, vel, veleval, dt, nsteps, K, weights=None, target=None):
    dev = torch.device("cuda:0")
    p0 = torch.from_numpy(np.ascontiguousarray(pos)).to(dev).requires_grad_()
    v0 = torch.from_numpy(np.ascontiguousarray(vel)).to(dev).requires_grad_()
    e0 = torch.from_numpy(np.ascontiguousarray(veleval)).to(dev).requires_grad_()
    mu = torch.tensor(float(system.params()[0].viscosity), dtype=torch.float64, requires_grad=True)
    pT = SPHRollout.apply(p0, v0, e0, mu, system, dt, nsteps, K)
    x = pT[:, :3].double()
    if weights is not None:
        loss = (x * torch.from_numpy(weights).to(dev)).sum()
    else:
        loss = ((x - torch.from_numpy(np.asarray(target, np.float64)[:, :3]).to(dev)) ** 2).sum(1).mean()
    loss.backward()
    return (p0.grad.cpu().numpy(), v0.grad.cpu().numpy(), e0.grad.cpu().numpy(), float(mu.grad.item()),
            pT.detach().cpu().numpy(), float(loss.item()))


def _check(label, got, want, floor, tol=1e-3):
    err = abs(got - want) / max(abs(want), floor)
    assert err <= tol, "%s: adjoint %.9e, FD %.9e, rel err %.3e" % (label, got, want, err)
    return err


def test_adjoint_short_rollout_matches_fd64():
    """Every input (pos, vel, veleval, viscosity) of a 5-step rollout with
    walls and friction active, against FP64 finite differences."""
    n, steps, K = 4096, 5, 2
    system, sp, g, gs = _system(n)
    pos, vel = dambreak(n, scene=3, velocity_sigma=0.3, velocity_seed=31)
    ve = np.zeros_like(vel)
    ve[:, :3] = normal(32, 3 * n, 0.2).reshape(n, 3)
    w = (2.0 * uniform(33, 3 * n) - 1.0).reshape(n, 3)
    gp, gv, ge, gmu, _, _ = _grads(system, pos, vel, ve, DT, steps, K, weights=w)
    coords, _ = sample_coordinates(n, 8, seed=34)
    errs = []
    for which, grad in (("pos", gp), ("vel", gv), ("veleval", ge)):
        scale = np.abs(grad[:, :3]).max()
        for (i, a) in coords:
            fd, same_branches, _ = fd_gradient(sp, gs, pos, vel, ve, DT, steps, which, (i, a), 1e-5, weights=w)
            if not same_branches:
                continue
            errs.append(_check("%s[%d,%d]" % (which, i, a), float(grad[i, a]), fd, 1e-2 * scale))
    fd, same_branches, _ = fd_gradient(sp, gs, pos, vel, ve, DT, steps, "visc", None, 1e-6, weights=w)
    assert same_branches
    errs.append(_check("viscosity", gmu, fd, 1e-12))
    assert len(errs) >= 20


def test_adjoint_checkpoint_interval_does_not_change_gradients():
    n, steps = 4096, 12
    system, sp, g, gs = _system(n)
    pos, vel = dambreak(n, scene=4, velocity_sigma=0.2, velocity_seed=41)
    ve = np.zeros_like(vel)
    w = (2.0 * uniform(42, 3 * n) - 1.0).reshape(n, 3)
    ref = None
    for K in (1, 5, 12, 100):
        gp, gv, ge, gmu, pT, _ = _grads(system, pos, vel, ve, DT, steps, K, weights=w)
        if ref is None:
            ref = (gp, gv, ge, gmu, pT)
            continue
        np.testing.assert_array_equal(pT, ref[4])
        np.testing.assert_array_equal(gp, ref[0])
        np.testing.assert_array_equal(gv, ref[1])
        np.testing.assert_array_equal(ge, ref[2])
        assert abs(gmu - ref[3]) <= 1e-9 * abs(ref[3])


def test_adjoint_backward_keeps_final_state_and_replays():
    """After the backward pass the context holds the rollout's final state and
    steps on exactly as if no gradient had been taken; a second backward pass
    gives the same gradients."""
    n, steps, K = 4096, 8, 3
    a, sp, g, gs = _system(n)
    b, _, _, _ = _system(n)
    pos, vel = dambreak(n, scene=5, velocity_sigma=0.2, velocity_seed=51)
    a.upload(pos, vel)
    b.upload(pos, vel)
    a.adjoint_record(DT, steps, K)
    b.step(DT, steps)
    dev = torch.device("cuda:0")
    gpos = torch.ones((n, 4), dtype=torch.float32, device=dev)
    out1 = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    out2 = torch.zeros_like(out1)
    torch.cuda.synchronize()  # the library runs on its own stream
    mu1 = a.adjoint_backward(dpos=gpos.data_ptr(), out_vel=out1.data_ptr())
    mu2 = a.adjoint_backward(dpos=gpos.data_ptr(), out_vel=out2.data_ptr())
    torch.cuda.synchronize()
    assert torch.equal(out1, out2)
    assert abs(mu1 - mu2) <= 1e-9 * abs(mu1)
    np.testing.assert_array_equal(a.get("pos_u", n), b.get("pos_u", n))
    np.testing.assert_array_equal(a.get("vel_u", n), b.get("vel_u", n))
    a.step(DT, 3)
    b.step(DT, 3)
    np.testing.assert_array_equal(a.get("pos_u", n), b.get("pos_u", n))


def test_adjoint_argument_and_state_errors():
    n = 1024
    system, sp, g, gs = _system(n)
    pos, vel = dambreak(n)
    system.upload(pos, vel)
    with pytest.raises(abi.SPHError) as e:
        system.adjoint_backward()
    assert e.value.code == abi.SPH_ESTATE
    with pytest.raises(abi.SPHError) as e:
        system.adjoint_record(DT, 0, 1)
    assert e.value.code == abi.SPH_EINVAL
    system.adjoint_record(DT, 4, 2)
    sp2 = system.params()[0]
    sp2.viscosity = 0.02
    system.updateParams(sp2)
    with pytest.raises(abi.SPHError) as e:
        system.adjoint_backward()
    assert e.value.code == abi.SPH_ESTATE
    # a particle thrown out of the grid: the rollout has no fixed particle set
    pos2, vel2 = pos.copy(), vel.copy()
    # 0.5 per step upwards: past the padded grid's top (z < 1.29) in 3 steps, where
    # the cell key exceeds nb_cells (an overflow in x would wrap to another row)
    vel2[0, :3] = (0.0, 0.0, 500.0)
    system.updateParams(sp)
    system.upload(pos2, vel2)
    with pytest.raises(abi.SPHError) as e:
        system.adjoint_record(DT, 6, 3)
    assert e.value.code == abi.SPH_EOOB


def _rollout_case_grads(n, steps, K, target_steps=None):
    pos, vel, vel_t, mu_t = rollout_case(n)
    tsys, _, _, _ = _system(n, viscosity=mu_t)
    tsys.upload(pos, vel_t)
    tsys.step(DT, steps if target_steps is None else target_steps)
    target = tsys.get("pos_u", n)
    tsys.close()
    system, sp, g, gs = _system(n)
    ve = np.zeros_like(vel)
    return (sp, gs, pos, vel, ve, target), _grads(system, pos, vel, ve, DT, steps, K, target=target)


def test_adjoint_rollout_case_matches_fd64():
    """The differentiable-rollout scene (65,536 particles, v0 ~ N(0, 0.1^2),
    loss = mean |x_T - x*|^2 against the rollout with viscosity 0.03 and
    perturbed v0, checkpoint every 20) over 50 steps: 32 random coordinates of
    dL/dv0 and dL/dviscosity against FP64 central differences (eps 1e-4),
    relative error <= 1e-3.

    50 steps is the horizon on which an FP32 rollout of this scene tracks the
    FP64 one (5e-7 apart); from about 75 steps on, particle pairs a fraction
    of a smoothing length apart amplify rounding differences and the FP32 and
    FP64 trajectories separate (0.5 h by step 200, the reference's own FP32
    arithmetic included), so no FP32 gradient can match an FP64 one there."""
    n, steps, K = 65536, 50, 20
    (sp, gs, pos, vel, ve, target), (gp, gv, ge, gmu, pT, loss) = _rollout_case_grads(n, steps, K)
    assert np.isfinite(gv).all() and np.isfinite(gmu)
    scale = np.abs(gv[:, :3]).max()
    checked, offset, errs, detail = 0, 0, [], []
    while checked < 32:
        coords, offset = sample_coordinates(n, 1, seed=13, offset=offset)
        (i, a), = coords
        fd, same_branches, _ = fd_gradient(sp, gs, pos, vel, ve, DT, steps, "vel", (i, a), 1e-4, target=target)
        if not same_branches:
            continue
        errs.append(_check("vel[%d,%d]" % (i, a), float(gv[i, a]), fd, 1e-3 * scale))
        detail.append((errs[-1], i, a, float(gv[i, a]), fd))
        checked += 1
    for e, i, a, got, want in sorted(detail, reverse=True)[:4]:
        print("  vel[%d,%d]: adjoint %.6e FD %.6e rel %.2e (|FD|/max|grad| %.2e)" % (i, a, got, want, e,
                                                                                     abs(want) / scale))
    # the viscosity moves every particle: shrink eps until no branch flips
    for eps in (1e-4, 1e-5, 1e-6, 1e-7):
        fd, same_branches, _ = fd_gradient(sp, gs, pos, vel, ve, DT, steps, "visc", None, eps, target=target)
        if same_branches:
            break
    assert same_branches, "no viscosity stencil free of branch changes"
    errs.append(_check("viscosity", gmu, fd, 1e-300))
    print("rollout case, %d steps: loss %.6e, max rel err %.3e over %d coordinates + viscosity (eps %.0e)"
          % (steps, loss, max(errs), checked, eps))


def test_adjoint_rollout_case_200_steps_checkpointing():
    """The full 200-step rollout: gradients are finite and do not depend on the
    checkpoint interval (K = 20 recomputes ten segments; K = 200 keeps the
    whole tape)."""
    n, steps = 65536, 200
    pos, vel, _, _ = rollout_case(n)
    ve = np.zeros_like(vel)
    w = (2.0 * uniform(14, 3 * n) - 1.0).reshape(n, 3) / n
    system, sp, g, gs = _system(n)
    res = [_grads(system, pos, vel, ve, DT, steps, K, weights=w) for K in (20, 200)]
    for r in res:
        assert np.isfinite(r[1]).all() and np.isfinite(r[3])
    np.testing.assert_array_equal(res[0][4], res[1][4])
    np.testing.assert_array_equal(res[0][1], res[1][1])
    np.testing.assert_array_equal(res[0][0], res[1][0])
    assert abs(res[0][3] - res[1][3]) <= 1e-9 * abs(res[1][3])
