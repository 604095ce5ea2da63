"""Batched differentiable rollout: every scene's gradients equal those of the
same scene in its own context, and batched gradient descent recovers hidden
per-scene viscosities."""
import numpy as np
import pytest
import torch

from enjaparticles_gb300 import abi
from enjaparticles_gb300.batch import Batch, dambreak_batch_scenes
from enjaparticles_gb300.calibrate import calibrate_viscosity, checkpoints, record_targets
from enjaparticles_gb300.scenes import dambreak, uniform
from enjaparticles_gb300.sph import SPH

pytestmark = pytest.mark.gpu

DT = 0.001


def _slot_tensor(batch, per_scene):
    """A (nslots, 4) float32 device tensor holding per_scene[s] at scene s's slots."""
    out = np.zeros((batch.nslots, 4), np.float32)
    for s, off in enumerate(batch.slot_offsets()):
        a = np.asarray(per_scene[s], np.float32)
        out[off:off + a.shape[0]] = a
    return torch.from_numpy(out).cuda()


def test_batch_adjoint_equals_lone_contexts():
    ns = [2048, 5000, 3333, 8192]
    mus = [0.005, 0.02, 0.035, 0.05]
    params = [abi.dambreak_params(n, mu) for n, mu in zip(ns, mus)]
    data = [dambreak(n, scene=10 + k, velocity_sigma=0.2, velocity_seed=60 + k) for k, n in enumerate(ns)]
    seeds = [(2.0 * uniform(70 + k, 4 * n) - 1.0).reshape(n, 4).astype(np.float32) for k, n in enumerate(ns)]
    for sd in seeds:
        sd[:, 3] = 0.0
    steps, K = 12, 5
    b = Batch(params, ns)
    for k, (pos, vel) in enumerate(data):
        b.upload(k, pos, vel)
    b.adjoint_record(DT, steps, K)
    gpos = _slot_tensor(b, seeds)
    out_p = torch.zeros_like(gpos)
    out_v = torch.zeros_like(gpos)
    out_e = torch.zeros_like(gpos)
    torch.cuda.synchronize()
    dmu = b.adjoint_backward(dpos=gpos.data_ptr(), out_pos=out_p.data_ptr(), out_vel=out_v.data_ptr(),
                             out_veleval=out_e.data_ptr())
    bp, bv, be = out_p.cpu().numpy(), out_v.cpu().numpy(), out_e.cpu().numpy()
    offs = b.slot_offsets()
    for k, ((sp, g, gs), (pos, vel), n) in enumerate(zip(params, data, ns)):
        s = SPH(sp, g, n, gs)
        s.upload(pos, vel)
        s.adjoint_record(DT, steps, K)
        np.testing.assert_array_equal(s.get("pos_u", n), b.get(k, "pos_u"))
        gp = torch.from_numpy(seeds[k]).cuda()
        op, ov, oe = torch.zeros_like(gp), torch.zeros_like(gp), torch.zeros_like(gp)
        torch.cuda.synchronize()
        mu_k = s.adjoint_backward(dpos=gp.data_ptr(), out_pos=op.data_ptr(), out_vel=ov.data_ptr(),
                                  out_veleval=oe.data_ptr())
        sl = slice(offs[k], offs[k] + n)
        np.testing.assert_array_equal(op.cpu().numpy()[:, :3], bp[sl, :3])
        np.testing.assert_array_equal(ov.cpu().numpy()[:, :3], bv[sl, :3])
        np.testing.assert_array_equal(oe.cpu().numpy()[:, :3], be[sl, :3])
        assert abs(mu_k - dmu[k]) <= 1e-9 * abs(mu_k), (k, mu_k, dmu[k])
        s.close()
    b.close()


def test_batch_loss_matches_numpy():
    ns = [1500, 4000]
    params = [abi.dambreak_params(n, 0.01) for n in ns]
    b = Batch(params, ns)
    data = [dambreak(n, scene=k) for k, n in enumerate(ns)]
    for k, (pos, vel) in enumerate(data):
        b.upload(k, pos, vel)
    tgt = [p + np.float32(0.01) * (2 * uniform(80 + k, 4 * p.shape[0]).reshape(-1, 4).astype(np.float32) - 1)
           for k, (p, _) in enumerate(data)]
    t = _slot_tensor(b, tgt)
    g = torch.zeros_like(t)
    torch.cuda.synchronize()
    losses = b.loss_mse(t.data_ptr(), g.data_ptr())
    gn = g.cpu().numpy()
    for k, ((pos, _), off) in enumerate(zip(data, b.slot_offsets())):
        d = pos[:, :3].astype(np.float64) - tgt[k][:, :3]
        assert abs(losses[k] - np.mean(np.sum(d * d, 1))) <= 1e-6 * losses[k]
        np.testing.assert_allclose(gn[off:off + ns[k], :3], 2 * d / ns[k], rtol=1e-5, atol=1e-12)
    b.close()


def test_batch_trajectory_backward_seeds_intermediate_times():
    """A loss gradient injected at checkpoint time 8 of a 12-step rollout gives
    the same initial-state gradients as the 8-step rollout seeded at its end."""
    ns = [3000, 6000]
    params = [abi.dambreak_params(n, mu) for n, mu in zip(ns, (0.01, 0.03))]
    data = [dambreak(n, scene=20 + k, velocity_sigma=0.2, velocity_seed=90 + k) for k, n in enumerate(ns)]
    b = Batch(params, ns)

    def load():
        for k, (pos, vel) in enumerate(data):
            b.upload(k, pos, vel)

    seed = _slot_tensor(b, [(2.0 * uniform(95 + k, 4 * n) - 1.0).reshape(n, 4) for k, n in enumerate(ns)])
    seed[:, 3] = 0
    load()
    b.adjoint_record(DT, 8, 4)
    v8 = torch.zeros_like(seed)
    torch.cuda.synchronize()
    mu8 = b.adjoint_backward(dpos=seed.data_ptr(), out_vel=v8.data_ptr())
    load()
    b.adjoint_record(DT, 12, 4)
    grads = torch.zeros((checkpoints(12, 4), b.nslots, 4), dtype=torch.float32, device="cuda")
    grads[2] = seed
    v12 = torch.zeros_like(seed)
    torch.cuda.synchronize()
    mu12 = b.adjoint_backward_traj(grads.data_ptr(), out_vel=v12.data_ptr())
    for k, (n, off) in enumerate(zip(ns, b.slot_offsets())):
        assert torch.equal(v8[off:off + n, :3], v12[off:off + n, :3])
        assert abs(mu8[k] - mu12[k]) <= 1e-9 * abs(mu8[k])
    b.close()


def test_batch_calibration_recovers_viscosity():
    """8 scenes with hidden viscosities: 30 batched gradient steps from 0.02
    on the trajectory loss."""
    S, steps, K = 8, 60, 10
    ns, _ = dambreak_batch_scenes(S, seed_n=21, n_lo=4096, n_hi=12000)
    hidden = [float(np.float32(0.005 + u * 0.045)) for u in uniform(22, S)]
    params = [abi.dambreak_params(n, 0.02) for n in ns]
    data = [dambreak(n, scene=k) for k, n in enumerate(ns)]
    b = Batch(params, ns)
    for k, (pos, vel) in enumerate(data):
        b.upload(k, pos, vel)
    targets = record_targets(b, hidden, steps, K, DT, torch)
    mu, hist = calibrate_viscosity(b, targets, [0.02] * S, iterations=30, nsteps=steps, K=K, dt=DT)
    err = np.abs(mu - np.asarray(hidden)) / np.asarray(hidden)
    print("calibration: hidden %s\n recovered %s\n rel err %s\n loss %s -> %s" % (
        np.round(hidden, 5), np.round(mu, 5), np.round(err, 4), hist[0][0], hist[-1][0]))
    assert np.max(err) < 0.05
    assert (hist[-1][0] <= hist[0][0]).all()
    b.close()
