#!/usr/bin/env python3
"""Benchmark: particle-updates/s of the 2,097,152-particle SPH dam break on GB300.

One step = hash+count -> tile totals -> cell scan -> place -> rank+permute -> density ->
velocity pass (beside density) -> force+collision+leapfrog over all particles (the fused path of sph_step,
replayed from a CUDA graph).  The workload is the 2M-particle configuration:
unit box, lattice spacing 2^-8, h = 2s, dt = 0.001, 1000-step rollout, seeded
synthetic dam-break lattice (no dataset exists for it).

  value  device-resident throughput over K steps (CUDA events on the
         library's stream, which is torch's current stream).
  e2e    the same metric through the C ABI with the state on the host: each
         step uploads pos/vel/veleval from pinned memory, steps, and
         downloads them again.
  roofline  the dominant kernel's algorithmic bytes / its mean duration
         (per-kernel CUDA events, sph_step_profile) against the measured
         HBM copy bandwidth.
  cpu_baseline  the CPU oracle (a port of the reference's kernels) on the
         host cores for a bounded sample.
  triangles  the same dam break with a 524-triangle mesh (collision_tri.cl
         after the walls): step time and the triangle stage's roofline.
  surface  SPH::postProcess on the 2M state: colour field and marching
         cubes at res 64 and 128.

`--impl reference` times the reference's CPU implementation instead: the
reference's OpenCL kernels cannot run on these machines (no OpenCL driver),
so its CPU stand-in is the oracle port, with all host threads.

Multi-GPU: the path does not shard (one scene per GPU): under torchrun every
rank runs its own replica, timing is max over ranks, value sums all ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT = 2097152
DT = 0.001
FALLBACK_HBM_GBS = 6800.0
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# the current kernels, from one ncu capture of the 2,097,152-particle dam break
# at the state named here; reported as roofline.traffic (with that state) for
# the dominant kernel at that workload.
TRAFFIC_STATE = "one launch at step 6 of the 2,097,152-particle dam break from the lattice at rest (ncu)"
MEASURED_TRAFFIC = {"k_force(fused collision+leapfrog)": 210.459904e6 + 71.135488e6,
                    "k_density": 94.924544e6 + 87.544064e6}
# The same captures' instruction-issue roofline, the bound these neighbour
# passes meet first: warp instructions (smsp__inst_executed.sum) over the 4
# an SM can issue per cycle in the launch's SM cycles (sm__cycles_elapsed.avg),
# on 152 SMs.
MEASURED_ISSUE = {"k_force(fused collision+leapfrog)": (222298374, 541018.80),
                  "k_density": (183728966, 456453.39)}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--exact", action="store_true", help="exact force arithmetic (bitwise oracle parity)")
    ap.add_argument("--e2e-steps", type=int, default=100)
    ap.add_argument("--profile-steps", type=int, default=0, help="0: same as --steps")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-seconds", type=float, default=120.0, help="time bound of the reference (CPU) arm")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batch-scenes", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=500)
    ap.add_argument("--serial-steps", type=int, default=10)
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-calibration", action="store_true")
    ap.add_argument("--cal-scenes", type=int, default=64)
    ap.add_argument("--cal-iters", type=int, default=50)
    ap.add_argument("--cal-steps", type=int, default=100)
    ap.add_argument("--cal-k", type=int, default=10)
    ap.add_argument("--adj-n", type=int, default=65536)
    ap.add_argument("--adj-steps", type=int, default=200)
    ap.add_argument("--adj-k", type=int, default=20)
    ap.add_argument("--no-triangles", action="store_true")
    ap.add_argument("--no-surface", action="store_true")
    ap.add_argument("--tri-steps", type=int, default=0, help="0: same as --steps")
    ap.add_argument("--steady-at", type=int, default=1000,
                    help="also time --steady-steps steps from this step of the rollout (0: skip)")
    ap.add_argument("--steady-steps", type=int, default=100)
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--dump-state", default=None,
                    help="step the dam break --dump-at steps from the lattice, save pos/vel/veleval (npz) and exit")
    ap.add_argument("--dump-at", type=int, default=1000)
    ap.add_argument("--init-state", default=None,
                    help="start the cfg1 sections from a state saved by --dump-state instead of the lattice")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def measured_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the GPU works."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "", 1).isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "", 1).isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        load = [v for v in sm if mx and v > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def algorithmic_bytes(n, c):
    """Compulsory bytes per step: one read of each input and one write of each
    output per stage of the reference's step, physics fields only (412N +
    24C), each stage's bytes given to the kernel that does that work:
      hash 24N -> count; the cell_start reset 4C and cellindices' 4C -> scan;
      sort 16N -> place; cellindices 4N + permute 100N -> permute (72N) and
      the velocity pass (32N: the veleval gather);
      density 20N+8C; force 68N+8C + collision 64N + leapfrog 116N -> force.
    The tile totals carry none."""
    return {"k_cell_count": 24.0 * n, "k_cell_totals": 0.0, "k_cell_scan": 8.0 * c, "k_cell_place": 16.0 * n,
            "k_cell_permute": 72.0 * n, "k_density": 20.0 * n + 8.0 * c, "k_step_velocities": 32.0 * n,
            "k_force(fused collision+leapfrog)": 248.0 * n + 8.0 * c}


def cpu_baseline_port(n, seconds):
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_bind
    from enjaparticles_gb300 import abi, scenes
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = scenes.dambreak(n)
    sim = oracle_bind.OracleSim(sp, g, gs, n)
    sim.upload(pos, vel)
    sim.step(DT, 1)  # warm-up
    steps, t0 = 0, time.perf_counter()
    while True:
        sim.step(DT, 1)
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds or steps >= 200:
            break
    threads = oracle_bind.oracle().oracle_threads()
    return {"value": n * steps / el, "unit": "particle-updates/s", "cores": threads, "kind": "port",
            "sample": "%d particles of the same dam-break rule, %d steps after 1 warm-up step, %.1f s" % (
                n, steps, el)}


def run_reference(args):
    """The reference arm: the reference's SPH step on the host cores, on the
    same 2,097,152-particle dam break.  The reference's own kernels are OpenCL
    and need an OpenCL driver, which these machines lack; they also compile
    for the host here (oracle/_ref) but only where the reference tree is, and
    x86 builds do not run on the Arm GPU hosts.  The oracle's port of those
    kernels (bit-identical to them on the host, all host threads) stands in.
    Each step is one full step of the whole system; the run stops after
    --steps steps or --ref-seconds seconds, whichever comes first."""
    rank, _, world = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_bind
    from enjaparticles_gb300 import scenes
    n = args.n
    # parameters derived by the oracle: this arm loads no library of the product
    sp, g, gs = oracle_bind.dambreak_params(n)
    pos, vel = scenes.dambreak(n)
    sim = oracle_bind.OracleSim(sp, g, gs, n)
    sim.upload(pos, vel)
    warm = min(args.warmup, 2)
    sim.step(DT, warm)
    steps, t0 = 0, time.perf_counter()
    while steps < args.steps:
        sim.step(DT, 1)
        steps += 1
        if time.perf_counter() - t0 >= args.ref_seconds:
            break
    el = time.perf_counter() - t0
    value = n * steps / el
    threads = oracle_bind.oracle().oracle_threads()
    line = {
        "metric": "particle-updates/s at 2M SPH", "value": value, "unit": "particle-updates/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * el / max(steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded dam-break lattice, zero initial velocity)",
        "config": config_block(n, g.nb_cells, warm, steps),
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "particle-updates/s", "cores": threads, "kind": "port",
                         "sample": "%d full SPH steps of the %d-particle dam break after %d warm-up steps (%.1f s; "
                                   "time-bounded at %.0f s) on %d host threads: the oracle's port of the "
                                   "reference's OpenCL kernels (bit-identical to them on the host)" % (
                                       steps, n, warm, el, args.ref_seconds, threads)},
        "e2e": {"value": value, "unit": "particle-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def bench_batched(args, torch):
    """The batched-scenes configuration: 256 dam breaks with N_s ~ U{2048..32768}
    (seed 7) and viscosity ~ U[0.005, 0.05], each with its own lattice, h and
    grid.  Batched: all scenes per step in one graph (sph_batch_step).  Serial:
    the same scenes, each in its own context, stepped one after the other
    (one graph launch per scene per step).  scenes/s = scenes * steps / time."""
    from enjaparticles_gb300 import abi, scenes
    from enjaparticles_gb300.batch import Batch, dambreak_batch_scenes
    from enjaparticles_gb300.sph import SPH
    import ctypes as C
    S = args.batch_scenes
    ns, mus = dambreak_batch_scenes(S)
    params = [abi.dambreak_params(n, mu) for n, mu in zip(ns, mus)]
    data = [scenes.dambreak(n, scene=k) for k, n in enumerate(ns)]
    stream = torch.cuda.current_stream()
    b = Batch(params, ns)
    b.set_stream(stream.cuda_stream)
    for k, (pos, vel) in enumerate(data):
        b.upload(k, pos, vel)
    b.step(DT, 5)
    b.sync()
    shape = list(b.launch_config()) if args.no_autotune else list(b.autotune(DT, steps=3))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    b.step(DT, args.batch_steps)
    e1.record(stream)
    e1.synchronize()
    t_batch = e0.elapsed_time(e1) / 1e3
    b.sync()
    # the same steps under the queue scheduler (persistent blocks over
    # (scene, tile) items), from the same starting state
    for k, (pos, vel) in enumerate(data):
        b.upload(k, pos, vel)
    b.set_scheduler(True)
    b.step(DT, 5)
    b.sync()
    torch.cuda.synchronize()
    e0.record(stream)
    b.step(DT, args.batch_steps)
    e1.record(stream)
    e1.synchronize()
    t_queue = e0.elapsed_time(e1) / 1e3
    b.sync()
    b.set_scheduler(False)
    deleted_last = b.out_of_grid()
    b.close()
    ctxs = []
    for (sp, g, gs), (pos, vel), n in zip(params, data, ns):
        s = SPH(sp, g, n, gs)
        abi.check(s.lib, s.ctx, s.lib.sph_set_stream(s.ctx, C.c_void_p(stream.cuda_stream)))
        s.upload(pos, vel)
        ctxs.append(s)
    for _ in range(2):
        for s in ctxs:
            s.step(DT, 1)
    if not args.no_autotune:  # the same tuner for the lone contexts (shapes change no result)
        for s in ctxs:
            s.autotune(DT, steps=2)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.serial_steps):
        for s in ctxs:
            s.step(DT, 1)
    e1.record(stream)
    e1.synchronize()
    t_serial = e0.elapsed_time(e1) / 1e3
    for s in ctxs:
        s.close()
    batched = S * args.batch_steps / t_batch
    serial = S * args.serial_steps / t_serial
    return {"metric": "scenes/s", "scenes": S, "particles": int(sum(ns)), "value": batched,
            "serial_value": serial, "speedup_vs_serial": batched / serial, "batch_steps": args.batch_steps,
            "serial_steps": args.serial_steps, "ms_per_batch_step": 1e3 * t_batch / args.batch_steps,
            "deleted_in_last_step": deleted_last,
            "launch_config": shape,
            "schedulers_ms_per_batch_step": {"grid": 1e3 * t_batch / args.batch_steps,
                                             "queue": 1e3 * t_queue / args.batch_steps},
            "note": "each scene of a batch steps bit-identically to the same scene in its own context"}


def bench_adjoint(args, torch):
    """The differentiable rollout: 65,536 particles of the dam-break lattice,
    v0 ~ N(0, 0.1^2), 200 steps, checkpoint every 20 steps.
      forward   200 plain steps (graph replays)
      record    the same 200 steps keeping the checkpoints (sph_adjoint_record)
      backward  segment recomputation + reverse kernels (sph_adjoint_backward,
                one graph), for a loss gradient on the final positions
    ratio = backward / forward (the adjoint step including its recomputation
    against the plain forward step)."""
    from enjaparticles_gb300 import abi, scenes
    from enjaparticles_gb300.sph import SPH
    import ctypes as C
    n, steps, K = args.adj_n, args.adj_steps, args.adj_k
    pos, vel, _, _ = scenes.rollout_case(n)
    sp, g, gs = abi.dambreak_params(n, 0.01)
    s = SPH(sp, g, n, gs)
    stream = torch.cuda.current_stream()
    abi.check(s.lib, s.ctx, s.lib.sph_set_stream(s.ctx, C.c_void_p(stream.cuda_stream)))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        torch.cuda.synchronize()
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1e3

    s.upload(pos, vel)
    s.step(DT, 10)
    s.upload(pos, vel)
    t_fwd = timed(lambda: s.step(DT, steps))
    dpos = torch.full((n, 4), 1.0 / n, dtype=torch.float32, device="cuda")
    dvel = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    s.upload(pos, vel)
    s.adjoint_record(DT, steps, K)
    t_build = timed(lambda: s.adjoint_backward(dpos=dpos.data_ptr(), out_vel=dvel.data_ptr()))
    t_rec, t_bwd = [], []
    for _ in range(3):
        s.upload(pos, vel)
        t_rec.append(timed(lambda: s.adjoint_record(DT, steps, K)))
        t_bwd.append(timed(lambda: s.adjoint_backward(dpos=dpos.data_ptr(), out_vel=dvel.data_ptr())))
    s.close()
    t_rec, t_bwd = min(t_rec), min(t_bwd)
    C1 = g.nb_cells + 1
    return {"metric": "adjoint/forward time", "particles": n, "steps": steps, "checkpoint_every": K,
            "forward_ms": 1e3 * t_fwd, "record_ms": 1e3 * t_rec, "backward_ms": 1e3 * t_bwd,
            "value": t_bwd / t_fwd, "record_plus_backward_over_forward": (t_rec + t_bwd) / t_fwd,
            "first_backward_ms_incl_graph_build": 1e3 * t_build,
            "tape_bytes": K * (132 * n + 8 * C1), "checkpoint_bytes": (steps // K + 2) * 48 * n}


def bench_calibration(args, torch):
    """Batched differentiable calibration: 64 dam-break scenes, N_s ~
    U{8192..65536} (seed 21), hidden viscosities mu_s ~ U[0.005, 0.05]
    (seed 22); targets = the final positions of 100-step runs with the hidden
    viscosities, kept at the checkpoint times; 50 batched gradient iterations
    on every mu_s from 0.02, each a 100-step recorded rollout (checkpoint every
    10 steps), the per-scene trajectory loss (mean squared distance at the 10
    checkpoint times) and one batched backward pass.  value = scenes *
    iterations / s over the whole loop."""
    import time
    import numpy as np
    from enjaparticles_gb300 import abi, scenes
    from enjaparticles_gb300.batch import Batch, dambreak_batch_scenes
    from enjaparticles_gb300.calibrate import calibrate_viscosity, record_targets
    S, steps = args.cal_scenes, args.cal_steps
    ns, _ = dambreak_batch_scenes(S, seed_n=21, n_lo=8192, n_hi=65536)
    hidden = [float(np.float32(0.005 + u * 0.045)) for u in scenes.uniform(22, S)]
    params = [abi.dambreak_params(n, mu) for n, mu in zip(ns, hidden)]
    data = [scenes.dambreak(n, scene=k) for k, n in enumerate(ns)]
    b = Batch(params, ns)
    b.set_stream(torch.cuda.current_stream().cuda_stream)
    for k, (pos, vel) in enumerate(data):
        b.upload(k, pos, vel)
    targets = record_targets(b, hidden, steps, args.cal_k, DT, torch)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    last = {}

    def keep_last(k, losses, mus, dmu):
        last["dmu"], last["mus"] = np.asarray(dmu, np.float64), np.asarray(mus, np.float64)

    mu, hist = calibrate_viscosity(b, targets, [0.02] * S, iterations=args.cal_iters, nsteps=steps, K=args.cal_k,
                                   dt=DT, on_iteration=keep_last)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    b.close()
    hidden = np.asarray(hidden)
    err = np.abs(mu - hidden)
    # the scenes recovered least well, with what the descent saw of them at
    # its last iteration: the loss (0 at the hidden viscosity, the targets
    # being that scene's own run) and its slope dL/dlog(mu)
    rel = err / hidden
    worst = []
    for s_ in np.argsort(rel)[::-1][:3]:
        worst.append({"scene": int(s_), "particles": int(ns[s_]), "hidden_mu": float(hidden[s_]),
                      "recovered_mu": float(mu[s_]), "rel_err": float(rel[s_]),
                      "loss_first": float(hist[0][0][s_]), "loss_last": float(hist[-1][0][s_]),
                      "dL_dlogmu_last": float(last["dmu"][s_] * last["mus"][s_]) if last else None})
    return {"metric": "scenes*iterations/s", "value": S * args.cal_iters / el, "scenes": S,
            "particles": int(sum(ns)), "iterations": args.cal_iters, "steps": steps, "checkpoint_every": args.cal_k,
            "seconds": el, "mu_abs_err_mean": float(err.mean()), "mu_abs_err_max": float(err.max()),
            "mu_rel_err_median": float(np.median(err / hidden)), "mu_rel_err_max": float((err / hidden).max()),
            "loss_first_median": float(np.median(hist[0][0])), "loss_last_median": float(np.median(hist[-1][0])),
            "start_mu": 0.02, "worst_scenes": worst,
            "note": "host wall clock around the whole loop (rollouts, losses, backward passes, iRprop- steps on log mu)"}


def bench_triangles(args, torch, peak):
    """Triangle-mesh collision (collision_tri.cl after the walls): the 2M
    dam break with the 524-triangle ramp-and-box mesh of
    scenes.ramp_and_box_mesh loaded (the ramp cuts through the fluid block).
      step   as many steps as the headline run of sph_step (the staged sequence with the
             triangle stage, replayed from a graph), CUDA events
      stage  sph_stage_collision_triangles alone (prep + contact kernels)
             over 50 launches on the state of the last step; its
             algorithmic bytes are 64 per particle (read position,
             velocity, force; write force) against the measured HBM copy
             bandwidth."""
    from enjaparticles_gb300 import abi, scenes
    from enjaparticles_gb300.sph import SPH
    import ctypes as C
    n = args.n
    sp, g, gs = abi.dambreak_params(n)
    pos0, vel0 = scenes.dambreak(n)
    tris = scenes.ramp_and_box_mesh()
    s = SPH(sp, g, n, gs)
    stream = torch.cuda.current_stream()
    abi.check(s.lib, s.ctx, s.lib.sph_set_stream(s.ctx, C.c_void_p(stream.cuda_stream)))
    s.loadTriangles(tris)
    s.upload(pos0, vel0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = args.tri_steps or args.steps
    s.step(DT, args.warmup)
    s.sync()
    e0.record(stream)
    s.step(DT, steps)
    e1.record(stream)
    e1.synchronize()
    t_step = e0.elapsed_time(e1) / steps
    reps = 50
    s.collision_triangles()
    s.sync()
    e0.record(stream)
    for _ in range(reps):
        abi.check(s.lib, s.ctx, s.lib.sph_stage_collision_triangles(s.ctx))
    e1.record(stream)
    e1.synchronize()
    t_stage = e0.elapsed_time(e1) / reps
    num = s.getNum()
    s.close()
    achieved = 64.0 * num / (t_stage / 1e3) / 1e9
    return {"metric": "particle-updates/s with a triangle mesh", "value": num * 1e3 / t_step,
            "unit": "particle-updates/s", "particles": num, "triangles": int(tris.shape[0]), "steps": steps,
            "ms_per_step": t_step, "stage_ms": t_stage,
            "stage_roofline": {"bound": "hbm", "algorithmic_bytes": 64 * num, "achieved": achieved, "peak": peak,
                               "unit": "GB/s", "frac": achieved / peak}}


def bench_surface(args, torch, peak):
    """SPH::postProcess on the 2M dam break after args.warmup + 100 steps:
    the colour field (res^3 samples, 27-cell walk) and marching cubes at
    isolevel 0.0001, at res 64 (the largest the reference's tiled image
    holds) and 128.  Device time per call (CUDA events, mean of 10), split
    into the colour field and the marching cubes (count, scan, emit; the
    count read back to the host in between).  Marching-cubes bytes: the field
    read by both passes plus the mesh written (72 B per triangle)."""
    from enjaparticles_gb300 import abi, scenes
    from enjaparticles_gb300.sph import SPH
    import ctypes as C
    n = args.n
    sp, g, gs = abi.dambreak_params(n)
    pos0, vel0 = scenes.dambreak(n)
    s = SPH(sp, g, n, gs)
    stream = torch.cuda.current_stream()
    abi.check(s.lib, s.ctx, s.lib.sph_set_stream(s.ctx, C.c_void_p(stream.cuda_stream)))
    s.upload(pos0, vel0)
    s.step(DT, args.warmup + 100)
    s.sync()
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    out = {}
    for res in (64, 128):
        ntri = C.c_int()
        abi.check(s.lib, s.ctx, s.lib.sph_post_process(s.ctx, res, C.byref(ntri)))
        t_cf = t_mc = 0.0
        reps = 10
        for _ in range(reps):
            e0.record(stream)
            abi.check(s.lib, s.ctx, s.lib.sph_colorfield(s.ctx, res))
            e1.record(stream)
            abi.check(s.lib, s.ctx, s.lib.sph_marching_cubes(s.ctx, None, res, 0.0001, C.byref(ntri)))
            e2.record(stream)
            e2.synchronize()
            t_cf += e0.elapsed_time(e1) / reps
            t_mc += e1.elapsed_time(e2) / reps
        mc_bytes = 2 * 4 * res ** 3 + 72 * ntri.value
        out["res%d" % res] = {"triangles": ntri.value, "colorfield_ms": t_cf, "marching_cubes_ms": t_mc,
                              "samples_per_s": res ** 3 / (t_cf / 1e3),
                              "mc_roofline": {"bound": "hbm", "algorithmic_bytes": mc_bytes,
                                              "achieved": mc_bytes / (t_mc / 1e3) / 1e9, "peak": peak,
                                              "unit": "GB/s", "frac": mc_bytes / (t_mc / 1e3) / 1e9 / peak}}
    s.close()
    out["particles"] = n
    out["state_after_steps"] = args.warmup + 100
    return out


def host_link(stream, pin, n, reps=10):
    """Copy rates of the host link on the e2e loop's own pinned buffers, with
    plain stream copies: the position upload (16 B per particle) that the step
    waits for, and the three state downloads (48 B per particle) that wait for
    the step.  The velocity uploads overlap the step and are not counted."""
    import torch

    dev = [torch.empty((n, 4), dtype=torch.float32, device="cuda") for _ in pin]
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    up = down = float("inf")
    for _ in range(reps):
        ev[0].record(stream)
        dev[0].copy_(pin[0], non_blocking=True)
        ev[1].record(stream)
        for d, h in zip(dev, pin):
            h.copy_(d, non_blocking=True)
        ev[2].record(stream)
        ev[2].synchronize()
        up = min(up, ev[0].elapsed_time(ev[1]))
        down = min(down, ev[1].elapsed_time(ev[2]))
    b = 16.0 * n
    return {"h2d_gbs": b / (up / 1e3) / 1e9, "d2h_gbs": len(pin) * b / (down / 1e3) / 1e9,
            "upload_pos_ms": up, "download_state_ms": down}


def config_block(n, c, warmup, steps):
    return {"workload": "SPH dam break, %d particles FP32, lattice spacing (0.125/N)^(1/3), h=2s, dt=0.001; "
                        "timed: steps %d..%d of the rollout from the lattice at rest" % (n, warmup, warmup + steps),
            "particles": n, "nb_cells": c, "dt": DT,
            "l2": "no flush: each step streams > 0.3 GB (> 129 MB L2)", "parallelism": "replicas (one scene per GPU)"}


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    rank, local_rank, world = dist_env()
    import torch
    torch.cuda.set_device(local_rank)
    from enjaparticles_gb300.replicas import Replicas
    reps = Replicas(device=torch.device("cuda", local_rank))
    from enjaparticles_gb300 import abi, scenes
    from enjaparticles_gb300.sph import SPH
    import ctypes as C

    n = args.n
    sp, g, gs = abi.dambreak_params(n)
    pos0, vel0 = scenes.dambreak(n)
    ve0 = np.zeros_like(pos0)
    s = SPH(sp, g, n, gs, exact=args.exact)
    lib = s.lib
    if args.init_state:
        # the scene's parameters and capacity stay those of args.n; the
        # particle count is the saved state's (particles may have left)
        st0 = np.load(args.init_state)
        pos0, vel0, ve0 = st0["pos"], st0["vel"], st0["veleval"]
        n = pos0.shape[0]
    if args.dump_state:
        # a later state of the same rollout, for profiling it without
        # stepping up to it under the profiler
        s.upload(pos0, vel0, ve0)
        s.step(DT, args.dump_at)
        s.sync()
        m = s.getNum()
        np.savez(args.dump_state, pos=s.get("pos_u", m), vel=s.get("vel_u", m), veleval=s.get("veleval_u", m))
        if reps.rank == 0:
            print(json.dumps({"dumped": args.dump_state, "steps": args.dump_at, "particles": m}))
        s.close()
        return
    # The library launches on this stream and the timing events are recorded
    # on it (a dedicated stream: the legacy default stream cannot host graphs).
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    abi.check(lib, s.ctx, lib.sph_set_stream(s.ctx, C.c_void_p(stream.cuda_stream)))

    barrier = reps.barrier
    max_over_ranks = reps.max

    sampler = ClockSampler(torch.cuda.current_device())
    # --- device-resident throughput (graph replay) --------------------------
    s.upload(pos0, vel0, ve0)
    s.step(DT, args.warmup)
    s.sync()
    # launch shapes: the autotuner times its candidates on this state (which
    # it restores) and keeps the fastest of each kernel
    launch = {"tuned": False, "shape": list(s.launch_config())}
    if not args.no_autotune:
        t0 = time.perf_counter()
        launch = {"tuned": True, "shape": list(s.autotune(DT, steps=3)),
                  "tuning_s": time.perf_counter() - t0}
    launch["keys"] = ["density_threads", "force_threads", "scan_tile_cells"]
    sampler.start()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s.step(DT, args.steps)
    e1.record(stream)
    e1.synchronize()
    barrier()
    t_ms = max_over_ranks(e0.elapsed_time(e1))
    s.sync()
    num_after = s.getNum()
    # --- per-kernel breakdown over the same trajectory ------------------------
    psteps = args.profile_steps or args.steps
    s.upload(pos0, vel0, ve0)
    s.step(DT, args.warmup)
    s.sync()
    cap = 16
    ms = (C.c_float * cap)()
    nk = C.c_int()
    phase = max(1, min(100, psteps))
    kname = [lib.sph_profile_kernel_name(s.ctx, k).decode() for k in range(cap)]
    i_force = next(k for k, nm in enumerate(kname) if nm.startswith("k_force"))
    i_density = kname.index("k_density")
    tot = None
    by_phase = []
    done = 0
    while done < psteps:
        k = min(phase, psteps - done)
        abi.check(lib, s.ctx, lib.sph_step_profile(s.ctx, DT, k, ms, cap, C.byref(nk)))
        row = [ms[q] for q in range(nk.value)]
        tot = row if tot is None else [a + b for a, b in zip(tot, row)]
        by_phase.append({"steps": [args.warmup + done, args.warmup + done + k], "ms_per_step": sum(row) / k,
                         "force_ms": row[i_force] / k, "density_ms": row[i_density] / k})
        done += k
    names = [lib.sph_profile_kernel_name(s.ctx, k).decode() for k in range(nk.value)]
    kern_ms = {names[k]: tot[k] / psteps for k in range(nk.value)}
    # --- end to end through the C ABI with host-resident state ----------------
    pin = [torch.empty((n, 4), dtype=torch.float32, pin_memory=True) for _ in range(3)]
    host = [p.numpy() for p in pin]
    host[0][:] = pos0
    host[1][:] = vel0
    host[2][:] = ve0
    f_pos, f_vel, f_ve = abi.FIELDS["pos_u"], abi.FIELDS["vel_u"], abi.FIELDS["veleval_u"]
    s.upload(host[0], host[1], host[2])
    s.step(DT, 3)
    s.sync()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        abi.check(lib, s.ctx, lib.sph_upload(s.ctx, host[0].ctypes.data, host[1].ctypes.data, host[2].ctypes.data, n))
        abi.check(lib, s.ctx, lib.sph_step(s.ctx, DT, 1))
        for fid, h in ((f_pos, host[0]), (f_vel, host[1]), (f_ve, host[2])):
            abi.check(lib, s.ctx, lib.sph_download_async(s.ctx, fid, h.ctypes.data, n))
        abi.check(lib, s.ctx, lib.sph_sync(s.ctx))
    t_e2e = max_over_ranks(time.perf_counter() - t0)
    barrier()
    link = host_link(stream, pin, n)
    # the device-resident step over the e2e loop's own window (its steps
    # start from the lattice), for the link floor below
    s.upload(pos0, vel0, ve0)
    s.sync()
    barrier()
    e0.record(stream)
    s.step(DT, args.e2e_steps)
    e1.record(stream)
    e1.synchronize()
    link["step_ms"] = max_over_ranks(e0.elapsed_time(e1)) / args.e2e_steps
    # --- the same step later in the rollout (the fluid has collapsed: more
    # neighbours per particle than near the lattice at rest) ------------------
    steady = None
    if args.steady_at > 0 and args.steady_steps > 0:
        s.upload(pos0, vel0, ve0)
        s.step(DT, args.steady_at)
        s.sync()
        barrier()
        e0.record(stream)
        s.step(DT, args.steady_steps)
        e1.record(stream)
        e1.synchronize()
        barrier()
        t_st = max_over_ranks(e0.elapsed_time(e1))
        s.sync()
        n_st = s.getNum()
        steady = {"steps": [args.steady_at, args.steady_at + args.steady_steps],
                  "ms_per_step": t_st / args.steady_steps,
                  "value": n_st * args.steady_steps * world / (t_st / 1e3), "unit": "particle-updates/s",
                  "particles": n_st}
    clocks = sampler.stop()

    steps = args.steps
    value = n * steps * world / (t_ms / 1e3)
    c = g.nb_cells
    ab = algorithmic_bytes(n, c)
    dom = max(kern_ms, key=lambda k: kern_ms[k])
    peak, peak_kind = measured_hbm()
    achieved = ab[dom] / (kern_ms[dom] / 1e3) / 1e9
    b_step = sum(ab.values())
    step_ms = t_ms / steps
    # the e2e loop's floor on this host link: the position upload, the step
    # (device-resident, the same steps) and the three downloads run one after
    # the other
    e2e_value = n * args.e2e_steps * world / t_e2e
    link["bound_value"] = n * world / ((link["upload_pos_ms"] + link["step_ms"] + link["download_state_ms"]) / 1e3)
    link["frac"] = e2e_value / link["bound_value"]
    line = {
        "metric": "particle-updates/s at 2M SPH", "value": value, "unit": "particle-updates/s", "n_gpus": world,
        "steps": steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded dam-break lattice, zero initial velocity)",
        "config": dict(config_block(n, c, args.warmup, steps),
                       **({"init_state": "%s (a saved later state of the same rollout; steps count from it)"
                           % args.init_state} if args.init_state else {})),
        "e2e": {"value": e2e_value, "unit": "particle-updates/s",
                "h2d_bytes_per_step": 3 * 16 * n, "d2h_bytes_per_step": 3 * 16 * n,
                "note": "state (pos, vel, veleval) uploaded from and downloaded to pinned host memory every step; "
                        "%d steps" % args.e2e_steps,
                "link": link},
        "gpu_launches": nk.value * steps,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "traffic": MEASURED_TRAFFIC.get(dom) if n == N_DEFAULT else None,
                     "traffic_state": TRAFFIC_STATE if n == N_DEFAULT else None, "peak_source": peak_kind,
                     "issue_frac": (MEASURED_ISSUE[dom][0] / (152 * 4 * MEASURED_ISSUE[dom][1])
                                    if n == N_DEFAULT and dom in MEASURED_ISSUE else None),
                     "algorithmic_bytes": ab[dom], "mean_launch_ms": kern_ms[dom]},
        "step_roofline": {"algorithmic_bytes": b_step, "achieved": b_step / (step_ms / 1e3) / 1e9, "peak": peak,
                          "frac": b_step / (step_ms / 1e3) / 1e9 / peak, "unit": "GB/s"},
        "steady_state": steady,
        "launch_config": launch,
        "kernels_ms": kern_ms,
        "kernels_by_phase": by_phase,
        "particles_after": num_after,
        "exact": bool(args.exact),
    }
    if clocks:
        line["clocks"] = clocks
    if rank == 0 and not args.no_batched:
        line["batched"] = bench_batched(args, torch)
    if rank == 0 and not args.no_adjoint:
        line["adjoint"] = bench_adjoint(args, torch)
    if rank == 0 and not args.no_triangles:
        line["triangles"] = bench_triangles(args, torch, peak)
    if rank == 0 and not args.no_surface:
        line["surface"] = bench_surface(args, torch, peak)
    if rank == 0 and not args.no_calibration:
        line["calibration"] = bench_calibration(args, torch)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_port(n, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line))
    s.close()
    reps.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
