"""Benchmark of the GB300 engine on the reference's headline workload.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--workload disk1m|plummer16k|plummer65k|plummer1m]

Workload (default, disk1m): the plain Barnes-Hut step with quadrupoles, theta 0.6, leaf <= 16,
N = 1e6 exponential disk (sech^2 vertical profile, scale height 0.1, R <= 10, disk mass 1, central
point mass 1), eps 0.005, dt 5e-4; one step = kick(dt/2), drift(dt), compute_forces, kick(dt/2)
through the engine's C ABI (the reference's lettuce-bench step, src/bench.cpp:174-181). Seeded
synthetic initial conditions; FP32 pair arithmetic, FP64 positions.

Prints one JSON line. value = mean device time per step (CUDA events on the engine stream, L2
flushed between steps outside the timed events); e2e = the same step through the public API with
host buffers: upload of the state from page-locked memory, the step, download of the state.
--impl reference times the reference CPU algorithm on the host's cores: the reference's own
backend when it was built here from its sources (oracle/_ref), else the CPU oracle port.
With --gpus N > 1 (torchrun) every rank runs an independent replica (the single-system step does
not shard without the multi-rank tree exchange, which is out of scope); value is the slowest rank.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms/step N=1e6 tree θ=0.6 at ≤1e-3 force err; adjoint÷forward, batched÷plain"

WORKLOADS = {
    "disk1m": dict(kind="disk", n=1_000_000, seed=1, eps=0.005, dt=5e-4, theta=0.6, method="tree",
                   desc="BH quadrupole tree, theta 0.6, leaf<=16, N=1e6 exponential disk (sech^2 h=0.1, R<=10, "
                        "core mass 1), eps 0.005, dt 5e-4"),
    "plummer16k": dict(kind="plummer", n=16384, seed=1, eps=0.01, dt=1e-3, theta=0.6, method="direct",
                       desc="direct summation, N=16384 Plummer (Henon units, r<10a), eps 0.01, dt 1e-3"),
    "plummer65k": dict(kind="plummer", n=65536, seed=2, eps=0.01, dt=1e-3, theta=0.6, method="direct",
                       desc="direct summation, N=65536 Plummer (Henon units, r<10a), eps 0.01, dt 1e-3"),
    "plummer1m": dict(kind="plummer", n=1_000_000, seed=1, eps=0.01, dt=1.0 / 128, theta=0.6, method="tree",
                      desc="BH quadrupole tree, theta 0.6, N=1e6 Plummer (Henon units, r<10a), eps 0.01, dt 1/128 "
                           "(the reference's published GPU configuration)"),
}


L2_NOTE = "flushed between timed steps (write of 2x L2 outside the step events)"


def workload_config(w, n, world):
    """The `config` object of both arms' lines (identical keys and values for the same workload)."""
    return {"workload": w["desc"], "n": n, "method": w["method"], "theta": w["theta"],
            "parallelism": "replicas" if world > 1 else "single-gpu", "l2": L2_NOTE}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return world, rank, local, dist
    return 1, 0, 0, None


def reduce_max(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def make_bodies(w):
    from lettuce_simulate_physics_gb300 import scenarios as S
    if w["kind"] == "disk":
        return S.disk(w["n"], w["seed"])
    return S.plummer(w["n"], w["seed"], cut=10.0)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def force_error_sample(be, b, w, count=256, seed=7):
    """Median and 99th-percentile per-body relative error of the engine's accelerations against an
    FP64 direct sum over all N bodies, for a seeded sample of bodies (numpy, chunked)."""
    a = be.accel()
    ids = be.download().id
    n = len(ids)
    rng = np.random.Generator(np.random.PCG64(seed))
    pick = rng.choice(n, size=min(count, n), replace=False)
    pos = be.pos64().T
    m = be.download().m.astype(np.float64)
    e2 = w["eps"] ** 2
    errs = []
    for s in range(0, len(pick), 8):
        idx = pick[s:s + 8]
        d = pos[None, :, :] - pos[idx][:, None, :]
        r2 = (d * d).sum(-1) + e2
        r2[np.arange(len(idx)), idx] = np.inf
        inv3 = r2 ** -1.5
        ref = (d * (m[None, :] * inv3)[..., None]).sum(1)
        got = a[:3, idx].T.astype(np.float64)
        errs.extend((np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)).tolist())
    return float(np.median(errs)), float(np.percentile(errs, 99))


def adjoint_leg(L, local, steps=1000, every=32, n=65536):
    """Adjoint of the direct-sum leapfrog at the configuration-2 shape: Plummer N=65536 (seed 2),
    eps 0.01, dt 1e-3, 1000 KDK steps, checkpoints every 32; target x* from a forward run whose
    initial positions carry Gaussian perturbations (sigma 1e-3). Returns forward and adjoint device
    milliseconds per step and their ratio."""
    from lettuce_simulate_physics_gb300 import scenarios as S
    be = L.CudaBackend(local)
    p = L.ForceParams(G=1.0, eps=0.01, method=L.ForceMethod.direct)
    dt = 1e-3
    b = S.plummer(n, 2, cut=10)
    rng = np.random.Generator(np.random.PCG64(2))
    bp = b.copy()
    bp.x += rng.normal(0, 1e-3, n).astype(np.float32)
    bp.y += rng.normal(0, 1e-3, n).astype(np.float32)
    bp.z += rng.normal(0, 1e-3, n).astype(np.float32)
    # Target: forward run of the perturbed initial conditions (plain steps).
    be.upload(bp)
    be.compute_forces(p, False)
    be.synchronize()
    be.event_record(2)
    for _ in range(steps):
        be.kick(0.5 * dt)
        be.drift(dt)
        be.compute_forces(p, False)
        be.kick(0.5 * dt)
    be.event_record(3)
    fwd_ms = be.event_elapsed(2, 3) / steps
    pos = be.pos64()
    ids = be.download().id
    xstar = np.zeros((n, 3))
    xstar[ids] = pos.T
    be.upload(b)
    be.synchronize()
    be.event_record(4)
    be.adjoint_forward(p, dt, steps, every)
    be.event_record(5)
    ck_fwd_ms = be.event_elapsed(4, 5) / steps
    be.event_record(6)
    loss, gx, gv, gm = be.adjoint_backward(xstar)
    be.event_record(7)
    adj_ms = be.event_elapsed(6, 7) / steps
    # The same with a checkpoint at every step: every position kept (steps x N x 44 B, 2.9 GB here),
    # so the backward pass needs no recomputation.
    be.upload(b)
    be.adjoint_forward(p, dt, steps, 1)
    be.synchronize()
    be.event_record(6)
    loss1, gx1, _, _ = be.adjoint_backward(xstar)
    be.event_record(7)
    adj1_ms = be.event_elapsed(6, 7) / steps
    be.close()
    return {"n": n, "steps": steps, "checkpoint_every": every, "loss": loss,
            "forward_ms_per_step": round(fwd_ms, 4), "checkpointed_forward_ms_per_step": round(ck_fwd_ms, 4),
            "adjoint_ms_per_step": round(adj_ms, 4), "adjoint_over_forward": round(adj_ms / fwd_ms, 3),
            # Against the forward step's device time alone (the checkpointed C++ loop, no host syncs):
            # the public-API loop above synchronises once per force call, which adds host time.
            "adjoint_over_device_forward": round(adj_ms / ck_fwd_ms, 3),
            "every_step_checkpoints": {"adjoint_ms_per_step": round(adj1_ms, 4),
                                       "adjoint_over_forward": round(adj1_ms / fwd_ms, 3),
                                       "same_gradient": bool(np.array_equal(gx, gx1))},
            "grad_norms": {"x": float(np.linalg.norm(gx)), "v": float(np.linalg.norm(gv)),
                           "m": float(np.linalg.norm(gm))}}


def fp64_direct_error(pos, m, acc, eps, count=64, seed=7):
    """Median and maximum per-body relative error of acc (n, 3) against an FP64 direct sum over
    all bodies (positions pos (n, 3), masses m), for a seeded sample of bodies."""
    n = len(m)
    rng = np.random.Generator(np.random.PCG64(seed))
    pick = rng.choice(n, size=min(count, n), replace=False)
    errs = []
    for s in range(0, len(pick), 16):
        idx = pick[s:s + 16]
        d = pos[None, :, :] - pos[idx][:, None, :]
        r2 = (d * d).sum(-1) + eps * eps
        r2[np.arange(len(idx)), idx] = np.inf
        ref = (d * (m[None, :] * r2 ** -1.5)[..., None]).sum(1)
        errs.extend((np.linalg.norm(acc[idx] - ref, axis=1) / np.linalg.norm(ref, axis=1)).tolist())
    return float(np.median(errs)), float(np.max(errs))


def ensemble_leg(L, local, steps=200, seq_steps=10, count=512):
    """Batched ensemble at the configuration-3 shape: 512 Plummer clusters (seeds 100-611), N
    log-uniform in [1024, 131072], eps = 0.01 (N/16384)^(-1/3), direct for N <= 8192 else tree
    theta 0.5, dt 1e-3, `steps` KDK steps as one CUDA graph (after the autotuner). Compared with
    the same systems run one at a time through the plain engine API (upload, then KDK steps with
    compute_forces), timed over `seq_steps` steps per system. Throughput in bodies x steps / s."""
    from lettuce_simulate_physics_gb300 import scenarios as S
    from lettuce_simulate_physics_gb300.ensemble import Ensemble
    b, counts, eps, theta, methods = S.ensemble(count)
    n = int(counts.sum())
    off = np.concatenate([[0], np.cumsum(counts.astype(np.int64))])
    dt = 1e-3
    en = Ensemble(local)
    en.upload(b, counts, eps, theta, methods)
    t0 = time.perf_counter()
    tun = en.tune()
    tune_s = time.perf_counter() - t0
    e0, _, _ = en.energy()
    # Force accuracy at t = 0 on four systems (smallest/largest direct and tree) vs FP64 direct.
    acc = en.accel()
    got = en.download()
    picks = []
    for meth in (0, 1):
        idx = np.flatnonzero(methods == meth)
        if len(idx):
            picks += [int(idx[np.argmin(counts[idx])]), int(idx[np.argmax(counts[idx])])]
    ferr = {}
    for k in picks:
        lo, hi = int(off[k]), int(off[k + 1])
        order = np.argsort(got.id[lo:hi])
        pos = np.stack([b.x[lo:hi], b.y[lo:hi], b.z[lo:hi]], 1).astype(np.float64)
        a = acc[:3, lo:hi].T[order].astype(np.float64)
        med, mx = fp64_direct_error(pos, b.m[lo:hi].astype(np.float64), a, float(eps[k]))
        ferr[f"sys{k}_N{hi - lo}_{'tree' if methods[k] else 'direct'}"] = {"median": med, "max": mx}
    # Batched: `steps` steps as one CUDA graph. The first run captures it (its energy change over
    # the configured 200 steps from t = 0 is the reported error); the timed run replays it.
    t0 = time.perf_counter()
    en.run(dt, steps, use_graph=True)
    first_wall = time.perf_counter() - t0
    e1, _, _ = en.energy()
    rel = np.abs((e1 - e0) / e0)
    t0 = time.perf_counter()
    en.run(dt, steps, use_graph=True)
    wall = time.perf_counter() - t0
    st = en.stats()
    en.close()
    batched_dev = n * steps / (st.run_ms * 1e-3)
    batched_wall = n * steps / wall
    # One at a time through the plain API.
    be = L.CudaBackend(local)
    seq_dev_ms = 0.0
    seq_wall_s = 0.0
    for k in range(len(counts)):
        lo, hi = int(off[k]), int(off[k + 1])
        sb = L.Bodies(b.x[lo:hi], b.y[lo:hi], b.z[lo:hi], b.vx[lo:hi], b.vy[lo:hi], b.vz[lo:hi], b.m[lo:hi],
                      b.id[lo:hi])
        p = L.ForceParams(G=1.0, eps=float(eps[k]), theta=float(theta[k]),
                          method=L.ForceMethod.tree if methods[k] else L.ForceMethod.direct)
        be.upload(sb)
        be.compute_forces(p, False)
        be.synchronize()
        t0 = time.perf_counter()
        be.event_record(8)
        for _ in range(seq_steps):
            be.kick(0.5 * dt)
            be.drift(dt)
            be.compute_forces(p, False)
            be.kick(0.5 * dt)
        be.event_record(9)
        be.synchronize()
        seq_wall_s += time.perf_counter() - t0
        seq_dev_ms += be.event_elapsed(8, 9)
    be.close()
    seq_dev = n * seq_steps / (seq_dev_ms * 1e-3)
    seq_wall = n * seq_steps / seq_wall_s
    return {
        "systems": int(len(counts)), "n_total": n, "n_tree_systems": int((methods == 1).sum()),
        "n_direct_systems": int((methods == 0).sum()), "steps": steps, "dt": dt,
        "tuning": {"direct_ipt": list(tun.direct_ipt), "direct_tile": list(tun.direct_tile), "walk_group": tun.walk_group, "tune_s": round(tune_s, 2)},
        "batched": {"run_ms": round(st.run_ms, 3), "wall_s": round(wall, 4), "used_graph": st.used_graph,
                    "recoveries": st.recoveries, "launches_per_step": st.launches_per_step,
                    "bodies_steps_per_s": batched_dev, "bodies_steps_per_s_wall": batched_wall,
                    "captures": st.captures, "first_run_wall_s": round(first_wall, 4)},
        "sequential": {"steps_per_system": seq_steps, "device_ms": round(seq_dev_ms, 3),
                       "wall_s": round(seq_wall_s, 4), "bodies_steps_per_s": seq_dev,
                       "bodies_steps_per_s_wall": seq_wall},
        "batched_over_sequential": round(batched_wall / seq_wall, 3),
        "batched_over_sequential_device": round(batched_dev / seq_dev, 3),
        "energy_rel_error": {"median": float(np.median(rel)), "p99": float(np.percentile(rel, 99)),
                             "max": float(np.max(rel)), "steps": steps},
        "force_error_vs_fp64_t0": ferr,
    }


def collision_leg(L, local, n_each=8_000_000, steps=500, adj_steps=64, every=8, radius=2.0, width=0.05, h=0.5):
    """Configuration 4: two inclined disks (each the disk1m recipe at n_each bodies) on a parabolic
    approach; tree theta 0.6, eps 0.005, dt 5e-4; `steps` plain KDK steps, the last `adj_steps` of
    them run as an adjoint window (frozen interaction lists, checkpoints every `every`). Loss: the
    disk-1 mass within `radius` of the disk-1 core at the end, smoothed with a logistic step of
    `width`; its gradient with respect to the disks' relative velocity at the start of the window
    (disk 1 moves by f1 dv, disk 2 by -f0 dv, f = mass fractions). The adjoint is checked against
    central differences of plain runs along the gradient with respect to all window-start
    velocities."""
    from lettuce_simulate_physics_gb300 import scenarios as S
    t0 = time.perf_counter()
    b, ne = S.collision(n_each)
    gen_s = time.perf_counter() - t0
    n = len(b)
    p = L.ForceParams(G=1.0, eps=0.005, theta=0.6, method=L.ForceMethod.tree)
    dt = 5e-4
    be = L.CudaBackend(local)
    be.upload(b)
    be.compute_forces(p, False)
    be.synchronize()
    pre = steps - adj_steps
    be.event_record(10)
    for _ in range(pre):
        be.kick(0.5 * dt)
        be.drift(dt)
        be.compute_forces(p, False)
        be.kick(0.5 * dt)
    be.event_record(11)
    fwd_ms = be.event_elapsed(10, 11) / max(pre, 1)
    bw = be.download()  # start of the adjoint window (positions rounded to float)
    m1 = float(bw.m[bw.id < ne].sum())
    m2 = float(bw.m[bw.id >= ne].sum())
    f1, f0 = m2 / (m1 + m2), m1 / (m1 + m2)
    d1 = np.zeros(n, bool)
    d1[:ne] = True

    def loss_and_seed(pos_by_id, m_by_id):
        c = pos_by_id[0]
        d = pos_by_id - c
        r = np.sqrt((d * d).sum(1))
        z = (radius - r) / width
        sig = 1.0 / (1.0 + np.exp(-z))
        Lv = float((m_by_id * sig)[d1].sum())
        coef = np.where(d1, m_by_id * sig * (1 - sig) / width, 0.0)
        coef[0] = 0.0
        g = -(coef / np.where(r > 0, r, 1.0))[:, None] * d
        g[0] -= g.sum(0)  # through the core's position
        return Lv, g

    def window(bodies):
        be.upload(bodies)
        be.compute_forces(p, False)
        for _ in range(adj_steps):
            be.kick(0.5 * dt)
            be.drift(dt)
            be.compute_forces(p, False)
            be.kick(0.5 * dt)
        ids = be.download().id
        pos = np.zeros((n, 3))
        pos[ids] = be.pos64().T
        return pos

    m_by_id = np.zeros(n)
    m_by_id[bw.id] = bw.m
    be.upload(bw)
    be.synchronize()
    be.event_record(12)
    be.adjoint_forward(p, dt, adj_steps, every)
    be.event_record(13)
    ids = be.download().id
    xT = np.zeros((n, 3))
    xT[ids] = be.pos64().T
    Lval, seed = loss_and_seed(xT, m_by_id)
    be.event_record(14)
    gx, gv, gm = be.adjoint_backward_seeded(seed)
    be.event_record(15)
    ck_ms = be.event_elapsed(12, 13) / adj_steps
    adj_ms = be.event_elapsed(14, 15) / adj_steps
    grad = f1 * gv[d1].sum(0) - f0 * gv[~d1].sum(0)
    # The relative-velocity gradient is tiny over the window (both disks translate almost rigidly,
    # the loss is measured about the disk-1 core), below what differences of FP32-force runs resolve.
    # The check is therefore along the full velocity gradient: plain runs from the same window start
    # with velocities moved by +-h gv/|gv| (lists rebuilt, not frozen), against |gv|.
    gnorm = float(np.linalg.norm(gv))
    u = gv / max(gnorm, 1e-300)
    lp, lm_ = [], []
    for sgn, out in ((1.0, lp), (-1.0, lm_)):
        bb = bw.copy()
        dv = sgn * h * u[bb.id]
        bb.vx = (bb.vx + dv[:, 0]).astype(np.float32)
        bb.vy = (bb.vy + dv[:, 1]).astype(np.float32)
        bb.vz = (bb.vz + dv[:, 2]).astype(np.float32)
        out.append(loss_and_seed(window(bb), m_by_id)[0])
    fd = (lp[0] - lm_[0]) / (2 * h)
    be.close()
    return {"n": n, "n_each": ne, "steps": steps, "adjoint_steps": adj_steps, "checkpoint_every": every,
            "generate_s": round(gen_s, 2), "forward_ms_per_step": round(fwd_ms, 3),
            "checkpointed_forward_ms_per_step": round(ck_ms, 3), "adjoint_ms_per_step": round(adj_ms, 3),
            "adjoint_over_forward": round(adj_ms / fwd_ms, 3),
            "loss": Lval, "dL_dvrel": grad.tolist(), "dL_dvrel_norm": float(np.linalg.norm(grad)),
            "velocity_gradient_norm": gnorm, "fd_along_velocity_gradient": fd,
            "fd_rel_diff": float(abs(fd - gnorm) / max(abs(fd), 1e-300)), "fd_step": h,
            "loss_radius": radius, "loss_width": width}


def direct_leg(L, local, steps=20, warmup=3, cpu_steps=5, no_cpu=False):
    """Direct summation at the plummer16k workload (N = 16384 Plummer, seed 1, r < 10a, eps 0.01,
    dt 1e-3): device milliseconds per KDK step and per force call (CUDA events on the engine stream,
    L2 flushed between steps outside the events), the direct kernel's roofline (20 flops per body
    pair over the pair-loop time, against the FFMA throughput measured on the same GPU), and the
    reference CPU algorithm on the host cores for the same step."""
    w = WORKLOADS["plummer16k"]
    b = make_bodies(w)
    n = len(b)
    be = L.CudaBackend(local)
    p = L.ForceParams(G=1.0, eps=w["eps"], theta=w["theta"], method=L.ForceMethod.direct)
    dt = w["dt"]

    def step():
        be.kick(0.5 * dt)
        be.drift(dt)
        be.compute_forces(p, False)
        be.kick(0.5 * dt)

    be.upload(b)
    be.compute_forces(p, False)
    for _ in range(max(warmup, 3)):
        step()
    be.synchronize()
    step_ms, force_ms, pair_ms = [], [], []
    for _ in range(steps):
        be.flush_l2()
        be.event_record(0)
        step()
        be.event_record(1)
        step_ms.append(be.event_elapsed(0, 1))
        t = be.times()
        force_ms.append(t.force_ms)
        pair_ms.append(t.walk_ms)
    peak = be.probe_fp32_peak()
    be.close()
    flops = 20.0 * n * (n - 1)
    achieved = statistics.fmean([flops / (t * 1e-3) / 1e12 for t in pair_ms])
    out = {"workload": w["desc"], "n": n, "steps": steps, "ms_per_step": round(statistics.fmean(step_ms), 4),
           "force_ms": round(statistics.fmean(force_ms), 4), "pair_loop_ms": round(statistics.fmean(pair_ms), 4),
           "ginteractions_per_s": round(n * (n - 1) / (statistics.fmean(force_ms) * 1e-3) / 1e9, 1),
           "roofline": {"bound": "fp32", "kernel": "direct", "achieved": round(achieved, 3), "peak": round(peak, 3),
                        "unit": "TFLOP/s", "frac": round(achieved / peak, 4) if peak else None,
                        "peak_source": "measured FFMA throughput on this GPU (lg_probe_fp32_peak)",
                        "flops_per_unit": {"body_pair": 20}}}
    if not no_cpu:
        cms, kind, threads, _ = cpu_port_steps(b, w, cpu_steps)
        out["cpu_baseline"] = {"value": round(cms, 3), "unit": "ms/step", "cores": threads, "kind": kind,
                               "sample": f"{cpu_steps} KDK steps of the full workload (N={n})"}
        out["cpu_over_gpu"] = round(cms / out["ms_per_step"], 1)
    return out


def engine_bench_loop(L, local, w, steps=20, warmup=3):
    """The engine timed exactly as baseline/ref_gpu.py times the reference's CUDA backend: the
    reference's lettuce-bench step (kick, drift, compute_forces, kick, then times(), which waits
    for the device), wall clock per step, no L2 flush; plus the engine's own phase split."""
    b = make_bodies(w)
    be = L.CudaBackend(local)
    method = L.ForceMethod.tree if w["method"] == "tree" else L.ForceMethod.direct
    p = L.ForceParams(G=1.0, eps=w["eps"], theta=w["theta"], method=method)
    dt = w["dt"]

    def step():
        be.kick(0.5 * dt)
        be.drift(dt)
        be.compute_forces(p, False)
        be.kick(0.5 * dt)
        return be.times()

    be.upload(b)
    be.compute_forces(p, False)
    err_med, err_max = force_error_sample(be, b, w)
    for _ in range(max(warmup, 1)):
        step()
    wall, force, inter = [], [], []
    for _ in range(steps):
        t0 = time.perf_counter()
        t = step()
        wall.append((time.perf_counter() - t0) * 1e3)
        force.append(t.force_ms)
        inter.append(t.interactions)
    be.close()
    return {"ms_per_step_wall": round(statistics.fmean(wall), 4),
            "median_ms_per_step_wall": round(statistics.median(wall), 4),
            "force_ms": round(statistics.fmean(force), 4), "interactions_per_step": int(statistics.fmean(inter)),
            "ginteractions_per_s": round(statistics.fmean(inter) / (statistics.fmean(force) * 1e-3) / 1e9, 2),
            "force_error_vs_fp64": {"median": err_med, "p99": err_max, "sample_bodies": 256}}


def reference_gpu_leg(L, local, names=("disk1m", "plummer1m"), steps=20, warmup=3):
    """The reference's own CUDA backend (src/cuda_backend.cu built unmodified for sm_103a, see
    baseline/) on the same GPU and the same bodies, against the engine timed the same way. The
    reference runs in a child process (baseline/ref_gpu.py), so a failure there cannot disturb the
    engine's measurements; its result, or its error, is reported."""
    out = {}
    for name in names:
        w = WORKLOADS[name]
        eng = engine_bench_loop(L, local, w, steps, warmup)
        cmd = [sys.executable, os.path.join(ROOT, "baseline", "ref_gpu.py"), "--workload", name, "--steps",
               str(steps), "--warmup", str(warmup), "--device", str(local)]
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
            lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
            ref = json.loads(lines[-1]) if r.returncode == 0 and lines else \
                {"error": f"exit {r.returncode}: {(r.stderr or r.stdout)[-600:]}"}
        except subprocess.TimeoutExpired:
            ref = {"error": "timed out after 900 s"}
        rec = {"workload": w["desc"], "reference": ref, "engine": eng}
        if "ms_per_step_wall" in ref:
            rec["speedup_step"] = round(ref["ms_per_step_wall"] / eng["ms_per_step_wall"], 3)
            rec["speedup_force"] = round(ref["phases_ms"]["force"] / eng["force_ms"], 3)
        out[name] = rec
    return out


def read_profile_traffic(workload):
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get(workload)
    except (OSError, ValueError):
        return None


def cpu_port_steps(b, w, steps, threads=0, warmup=0, budget_s=None):
    """The reference CPU algorithm (oracle/_ref if built from the reference, else the port): one
    force call, `warmup` untimed KDK steps, then up to `steps` timed KDK steps; with a budget, the
    timed steps stop once they have used budget_s seconds (at least one runs). Returns (ms/step,
    kind, threads, timed steps)."""
    from oracle import oracle as O
    O.build()
    kind = "ref" if O.available("ref") else "port"
    cpu = O.OracleBackend(kind, threads)
    method = O.TREE if w["method"] == "tree" else O.DIRECT

    def step():
        cpu.kick(0.5 * w["dt"])
        cpu.drift(w["dt"])
        cpu.compute_forces(method, 1.0, w["eps"], w["theta"], False)
        cpu.kick(0.5 * w["dt"])

    cpu.upload(b)
    cpu.compute_forces(method, 1.0, w["eps"], w["theta"], False)
    for _ in range(warmup):
        step()
    done = 0
    t0 = time.perf_counter()
    while done < max(steps, 1):
        step()
        done += 1
        if budget_s is not None and time.perf_counter() - t0 >= budget_s:
            break
    ms = (time.perf_counter() - t0) * 1e3 / done
    nt = cpu.threads()
    cpu.close()
    return ms, ("reference" if kind == "ref" else "port"), int(nt), done


def run_reference(args, w, world, rank, dist):
    if rank != 0:
        return 0
    b = make_bodies(w)
    steps = max(1, args.steps)
    # The full-N step, W untimed and K timed like the GPU arm; the timed steps stop early only if
    # they exceed the time budget (a few minutes in all).
    ms, kind, threads, done = cpu_port_steps(b, w, steps, warmup=max(0, args.warmup), budget_s=args.ref_budget_s)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(ms, 3), "unit": "ms/step", "n_gpus": args.gpus,
        "steps": done, "warmup": max(0, args.warmup), "ms_per_step": round(ms, 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32-pairs/f32-positions", "data": "synthetic (seeded)",
        "config": workload_config(w, w["n"], world),
        "cpu_baseline": {"value": round(ms, 3), "unit": "ms/step", "cores": threads, "kind": kind,
                         "sample": f"{done} timed KDK steps of the full workload (N={w['n']}) after one force call "
                                   f"and {max(0, args.warmup)} untimed steps"},
        "e2e": {"value": round(ms, 3), "unit": "ms/step", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# Algorithmic bytes per body of the tree step's memory-side phases (this engine's layout):
#   sort:  bounding box (read FP64 x, y, z: 24), keys (read 24, write key 8 + index 4), histogram
#          (read keys 8), eight onesweep passes (read and write key + index: 24 each), permute (read
#          and write the body arrays, 81 B each way, plus the index 4);
#   build: keys read once (8), positions and masses read once by the leaf moments (32), node
#          records written once (about N/4 nodes x 96 B: range, geometry, moments).
SORT_BYTES_PER_BODY = 24 + 36 + 8 + 8 * 24 + 2 * 81 + 4
BUILD_BYTES_PER_BODY = 8 + 32 + 24


def hbm_peak():
    """(GB/s, source): the measured copy bandwidth of the GB300s, else the fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def phase_roofline(n, sort_ms, build_ms):
    peak, src = hbm_peak()
    out = {}
    for name, per, t in (("sort", SORT_BYTES_PER_BODY, sort_ms), ("build", BUILD_BYTES_PER_BODY, build_ms)):
        gbs = n * per / (t * 1e-3) / 1e9 if t > 0 else None
        out[name] = {"bound": "hbm", "bytes_per_body": per, "achieved": round(gbs, 1) if gbs else None,
                     "peak": peak, "unit": "GB/s", "frac": round(gbs / peak, 4) if gbs else None,
                     "peak_source": src}
    out["build"]["note"] = ("FP64-latency bound in practice: the moments upsweep (leaf moments and one "
                            "launch per tree level) is about half of the phase")
    out["sort"]["note"] = "eight dependent onesweep passes, each limited by its decoupled look-back"
    return out


def run_gb300(args, w, world, rank, local, dist):
    import lettuce_simulate_physics_gb300 as L
    from lettuce_simulate_physics_gb300 import build as B
    from lettuce_simulate_physics_gb300.backend import PinnedBodies
    B.build()
    b = make_bodies(w)
    n = len(b)
    be = L.CudaBackend(local)
    method = L.ForceMethod.tree if w["method"] == "tree" else L.ForceMethod.direct
    p = L.ForceParams(G=1.0, eps=w["eps"], theta=w["theta"], method=method)
    dt = w["dt"]
    be.upload(b)
    be.compute_forces(p, False)
    err_med, err_p99 = force_error_sample(be, b, w)

    def step():
        be.kick(0.5 * dt)
        be.drift(dt)
        be.compute_forces(p, False)
        be.kick(0.5 * dt)

    for _ in range(max(args.warmup, 3)):
        step()
    be.synchronize()
    walk_ms, sort_ms, build_ms, force_ms, step_ms, inter, pairs, cells = [], [], [], [], [], [], [], []
    barrier(dist)
    launches0 = be.launch_count()
    with ClockSampler(local) as clk:
        be.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            be.flush_l2()
            be.event_record(0)
            step()
            be.event_record(1)
            step_ms.append(be.event_elapsed(0, 1))
            t = be.times()
            walk_ms.append(t.walk_ms)
            sort_ms.append(t.sort_ms)
            build_ms.append(t.build_ms)
            force_ms.append(t.force_ms)
            inter.append(t.interactions)
            bp, ct = be.interaction_split()
            pairs.append(bp)
            cells.append(ct)
        be.synchronize()
        wall = time.perf_counter() - t0
        launches = be.launch_count() - launches0
        # The same step under load for a few hundred milliseconds more, so that the 200 ms clock
        # samples cover the step (not timed).
        t1 = time.perf_counter()
        while time.perf_counter() - t1 < 0.6:
            step()
            be.synchronize()
    barrier(dist)
    ms = reduce_max(dist, statistics.fmean(step_ms))
    clocks = clk.summary()

    # Roofline of the dominant kernel (the walk): algorithmic flops / walk time.
    # 20 flops per body-body pair, 65 per quadrupole cell term (the GRAPE-style per-unit counts).
    if method == L.ForceMethod.tree:
        flops = [20.0 * a + 65.0 * c for a, c in zip(pairs, cells)]
    else:
        flops = [20.0 * a for a in pairs]
    achieved = statistics.fmean([f / (t_ms * 1e-3) / 1e12 for f, t_ms in zip(flops, walk_ms)])
    peak = be.probe_fp32_peak()
    traffic = read_profile_traffic(args.workload)

    # End to end through the public API with host buffers: upload from page-locked memory, one
    # step, download of the state into page-locked memory, each step.
    pin, pin_out = PinnedBodies(n), PinnedBodies(n)
    hb = pin.bodies
    for f in ("x", "y", "z", "vx", "vy", "vz", "m", "id"):
        getattr(hb, f)[:] = getattr(b, f)
    e2e_steps = max(1, min(args.steps, 10))
    be.upload(hb)
    be.compute_forces(p, False)
    be.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        be.upload(hb)
        be.compute_forces(p, False)
        step()
        be.download(pin_out.bodies)
    e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
    pin.free()
    pin_out.free()
    e2e_ms = reduce_max(dist, e2e_ms)

    # CPU baseline (rank 0, N=1): the reference CPU algorithm on this host's cores, bounded sample.
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cms, kind, threads, _ = cpu_port_steps(b, w, args.ref_steps)
        cpu = {"value": round(cms, 3), "unit": "ms/step", "cores": threads, "kind": kind,
               "sample": f"{args.ref_steps} KDK step(s) of the full workload (N={n}) after one warm-up force call"}

    adj = None
    if rank == 0 and not args.no_adjoint:
        adj = adjoint_leg(L, local, steps=args.adjoint_steps, n=args.adjoint_n)

    ens = None
    if rank == 0 and not args.no_ensemble:
        ens = ensemble_leg(L, local, steps=args.ensemble_steps, count=args.ensemble_count)

    direct = None
    if rank == 0 and not args.no_direct:
        direct = direct_leg(L, local, no_cpu=args.no_cpu or world > 1)

    refgpu = None
    if rank == 0 and not args.no_reference_gpu:
        refgpu = reference_gpu_leg(L, local)

    coll = None
    if rank == 0 and not args.no_collision:
        coll = collision_leg(L, local, n_each=args.collision_n, steps=args.collision_steps,
                             adj_steps=args.collision_adj_steps, every=args.collision_every)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(ms, 4), "unit": "ms/step", "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": round(ms, 4), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32-pairs/f64-positions", "data": "synthetic (seeded)",
            "config": workload_config(w, n, world),
            "phases_ms": {"sort": round(statistics.fmean(sort_ms), 4), "build": round(statistics.fmean(build_ms), 4),
                          "walk": round(statistics.fmean(walk_ms), 4), "force": round(statistics.fmean(force_ms), 4)},
            "interactions_per_step": int(statistics.fmean(inter)),
            "ginteractions_per_s": round(statistics.fmean(inter) / (statistics.fmean(force_ms) * 1e-3) / 1e9, 2),
            "force_error_vs_fp64": {"median": err_med, "p99": err_p99, "sample_bodies": 256},
            "phase_roofline": phase_roofline(n, statistics.fmean(sort_ms), statistics.fmean(build_ms))
            if method == L.ForceMethod.tree else None,
            "roofline": {"bound": "fp32", "kernel": "walk" if method == L.ForceMethod.tree else "direct",
                         "achieved": round(achieved, 3), "peak": round(peak, 3), "unit": "TFLOP/s",
                         "frac": round(achieved / peak, 4) if peak else None, "traffic": traffic,
                         "peak_source": "measured FFMA throughput on this GPU (lg_probe_fp32_peak)",
                         "flops_per_unit": {"body_pair": 20, "cell_term": 65}},
            "cpu_baseline": cpu,
            "direct_c0": direct,
            "reference_gpu": refgpu,
            "adjoint": adj,
            "ensemble": ens,
            "collision": coll,
            "e2e": {"value": round(e2e_ms, 3), "unit": "ms/step", "h2d_bytes_per_step": 32 * n,
                    "d2h_bytes_per_step": 32 * n},
            "gpu_launches": int(launches),
            "clocks": clocks,
            "wall_s": round(wall, 3),
        }
        print(json.dumps(line), flush=True)
    be.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="disk1m", choices=sorted(WORKLOADS))
    ap.add_argument("--ref-steps", type=int, default=2, help="KDK steps of the CPU baseline leg of the GPU arm")
    ap.add_argument("--ref-budget-s", type=float, default=150.0,
                    help="--impl reference: time budget of its timed steps (stops early past it)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint leg")
    ap.add_argument("--adjoint-steps", type=int, default=1000, help="KDK steps of the adjoint leg")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the batched-ensemble leg")
    ap.add_argument("--ensemble-steps", type=int, default=200, help="KDK steps of the ensemble leg")
    ap.add_argument("--no-collision", action="store_true", help="skip the two-disk collision leg (adjoint window)")
    ap.add_argument("--no-direct", action="store_true", help="skip the direct-summation (plummer16k) leg")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip the reference CUDA backend on the same GPU (disk1m and plummer1m)")
    ap.add_argument("--collision-n", type=int, default=8_000_000, help="bodies per disk of the collision leg")
    ap.add_argument("--collision-steps", type=int, default=500, help="KDK steps of the collision leg")
    ap.add_argument("--collision-adj-steps", type=int, default=64, help="adjoint window of the collision leg")
    ap.add_argument("--collision-every", type=int, default=8, help="checkpoint interval of the collision window")
    ap.add_argument("--adjoint-n", type=int, default=65536, help="bodies of the adjoint leg")
    ap.add_argument("--ensemble-count", type=int, default=512, help="systems of the ensemble leg")
    ap.add_argument("--only", choices=["adjoint", "ensemble", "collision", "direct", "reference_gpu"],
                    help="run one leg alone (single GPU) and print its JSON result")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    if args.only:
        import lettuce_simulate_physics_gb300 as L
        from lettuce_simulate_physics_gb300 import build as B
        B.build()
        if args.only == "adjoint":
            out = adjoint_leg(L, 0, steps=args.adjoint_steps, n=args.adjoint_n)
        elif args.only == "ensemble":
            out = ensemble_leg(L, 0, steps=args.ensemble_steps, count=args.ensemble_count)
        elif args.only == "direct":
            out = direct_leg(L, 0, no_cpu=args.no_cpu)
        elif args.only == "reference_gpu":
            out = reference_gpu_leg(L, 0)
        else:
            out = collision_leg(L, 0, n_each=args.collision_n, steps=args.collision_steps,
                                adj_steps=args.collision_adj_steps, every=args.collision_every)
        print(json.dumps({"leg": args.only, **out}), flush=True)
        return 0
    world, rank, local, dist = dist_setup()
    if args.impl == "reference":
        return run_reference(args, w, world, rank, dist)
    return run_gb300(args, w, world, rank, local, dist)


if __name__ == "__main__":
    sys.exit(main())
