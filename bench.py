#!/usr/bin/env python3
"""Benchmark of the blobs step on GB300: sphere-steps/s of a 1,000,000-sphere
world (Physics::step = 8 substeps at dt = 1/120, r ~ U[0.05, 0.15], 40%
packing with overlaps, walled box, seeded synthetic scene, 1,000-step
rollout).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
  python bench.py --section general|batched|dense [--steps K] [--warmup W]

One JSON line on rank 0.  The whole 1,000-step rollout runs from t = 0,
every step between its own CUDA-event pair on the world's stream with L2
flushed before it (inputs resident in HBM); `value` is over K steps evenly
spaced across steps W .. 999 (a stratified sample of the rollout, whose
contact load grows along it), `rollout` over all 1,000.  The phase-timing,
roofline and end-to-end legs reload the scene and time the same K steps.
`e2e` is the same metric through the C ABI with the body state written from
and read back into pinned host memory every step; `roofline` is the step
kernel's algorithmic bytes per launch over its event-timed duration (events
around that kernel alone); `cpu_baseline` is the oracle (the CPU restatement
of the reference step) on bounded samples of the same workload, extrapolated
with the reference's O(N^2) cost model.  Secondary workloads follow: the
1,000-sphere world in full on GPU and CPU, the 4,096 batched worlds, the
differentiable batch, the jointed world, the literal 2000 x 2000 box.
With --gpus N > 1 (torchrun) every rank steps its own independent world
(replicas; the path has no data exchange).  --section runs one secondary
workload alone (the 200k-body jointed world, or the 4,096 batched worlds)
with per-phase timing: the driver of the launch lists under profiles/.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# algorithmic bytes (the minimal traffic model of the path)
BYTES_PER_BODY_SUBSTEP = 56      # state 40 B (read pos, pos_old, radius, mass; write pos, pos_old) + broadphase 16 B
BYTES_CONTACT_PER_BODY = 48      # fused contact+integrate: state 40 B + read back cell key + index 8 B
BYTES_PER_SPRING_SUBSTEP = 20    # a, b, rest, k, c
FALLBACK_HBM_GBS = 6800.0


def peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def profile_traffic(name):
    """dram bytes per launch from a committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(p):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


class Clocks:
    """nvidia-smi sampler over the timed region (read-only queries)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None
        self.skip = 0

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            # the timed region starts once the sampler is running
            t0 = time.time()
            while time.time() - t0 < 5.0 and os.path.getsize(self.path) == 0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.skip = sum(1 for _ in open(self.path))
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = list(open(self.path))
        # samples taken inside the timed region (the ones before it are dropped,
        # unless the region was shorter than the sampling interval)
        lines = lines[self.skip:] or lines[-1:]
        for line in lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle on samples of the workload
# ---------------------------------------------------------------------------
def cpu_baseline(sizes=(4096, 8192, 16384, 32768), target_n=1_000_000, seed=2, steps_per_size=1):
    """Times Physics::step of the f32 oracle (single thread, with the
    reference's per-body spatial-hash maintenance) on worlds of the same
    density, fits t(N) = a N^2 + b N and extrapolates to target_n."""
    import numpy as np
    from blobs_gb300 import scenes
    from oracle import oracle
    ns, ts = [], []
    for n in sizes:
        s = scenes.dense_spheres(seed=seed, n=n)
        w = oracle.OracleWorld(s, 32, maintain_spatial_hash=True)
        w.time_steps(s.dt, 1)  # first step: pending velocity requests
        t = w.time_steps(s.dt, steps_per_size) / steps_per_size
        ns.append(n)
        ts.append(t)
    A = np.array([[n * n, n] for n in ns], float)
    coef, *_ = np.linalg.lstsq(A, np.array(ts), rcond=None)
    t_target = float(coef[0] * target_n * target_n + coef[1] * target_n)
    return {
        "value": target_n / t_target,
        "unit": "sphere-steps/s",
        "cores": 1,
        "kind": "port",
        "sample": "oracle Physics::step on %s-sphere worlds of the same density (1 step each, %.1f s total), fit "
                  "t = a N^2 + b N, extrapolated to N=%d: %.1f s/step" % ("/".join(str(n) for n in ns), sum(ts),
                                                                         target_n, t_target),
        "cpu": platform.processor() or platform.machine(),
    }


def _fit_quadratic(ns, ts):
    """Least-squares t(N) = a N^2 + b N (the reference's C^2/2 pair loop
    plus per-body work)."""
    import numpy as np
    A = np.array([[n * n, n] for n in ns], float)
    coef, *_ = np.linalg.lstsq(A, np.array(ts), rcond=None)
    return float(coef[0]), float(coef[1])


def cpu_general(sizes=(2000, 4000, 8000), target_n=200_000, seed=3):
    """The oracle step on jointed worlds of the same density (side scaled
    with sqrt(N), joints N/4, springs N/2), fitted and extrapolated to the
    200k-body world."""
    from blobs_gb300 import scenes
    from oracle import oracle
    ns, ts = [], []
    for n in sizes:
        s = scenes.jointed_bodies(seed=seed, n=n, n_joints=n // 4, n_springs=n // 2,
                                  side=1500.0 * (n / 200_000.0) ** 0.5)
        w = oracle.OracleWorld(s, 32, maintain_spatial_hash=True)
        w.time_steps(s.dt, 1)
        ns.append(n)
        ts.append(w.time_steps(s.dt, 1))
    a, b = _fit_quadratic(ns, ts)
    t = a * target_n * target_n + b * target_n
    return {"value": target_n / t, "unit": "body-steps/s", "cores": 1, "kind": "port",
            "sample": "oracle Physics::step on %s-body jointed worlds of the same density (1 step each, %.1f s), "
                      "fit t = a N^2 + b N, extrapolated to N=%d: %.1f s/step"
                      % ("/".join(map(str, ns)), sum(ts), target_n, t)}


def cpu_batched(scene, sample=48):
    """The oracle step on `sample` worlds of the uneven batch (evenly spaced
    by index), fitted t(N) = a N^2 + b N over their body counts and summed
    over all worlds' body counts: one CPU step of the whole batch."""
    import numpy as np
    from blobs_gb300 import scenes
    from oracle import oracle
    idx = np.linspace(0, scene.n_worlds - 1, sample).astype(int)
    ns, ts = [], []
    for i in idx:
        sub = scenes.unpack_world(scene, int(i))
        w = oracle.OracleWorld(sub, 32, maintain_spatial_hash=True)
        w.time_steps(scene.dt, 1)
        ns.append(sub.n_bodies)
        ts.append(w.time_steps(scene.dt, 1))
    a, b = _fit_quadratic(ns, ts)
    counts = np.diff(scene.world_body_offsets).astype(np.float64)
    t = float(np.sum(a * counts * counts + b * counts))
    return {"value": scene.n_bodies / t, "unit": "sphere-steps/s", "cores": 1, "kind": "port",
            "sample": "oracle Physics::step on %d evenly spaced worlds (%d-%d bodies, %.1f s), fit t = a N^2 + b N, "
                      "summed over all %d worlds: %.2f s per batch step"
                      % (sample, min(ns), max(ns), sum(ts), scene.n_worlds, t)}


def cpu_gradient_batch(scene, sample=4):
    """The oracle forward step on `sample` of the 256 equal worlds, scaled
    by the world count (the reference has no backward pass)."""
    import numpy as np
    from blobs_gb300 import scenes
    from oracle import oracle
    ts = []
    for i in np.linspace(0, scene.n_worlds - 1, sample).astype(int):
        sub = scenes.unpack_world(scene, int(i))
        w = oracle.OracleWorld(sub, 32, maintain_spatial_hash=True)
        w.time_steps(scene.dt, 1)
        ts.append(w.time_steps(scene.dt, 1))
    t = float(np.mean(ts)) * scene.n_worlds
    return {"value": scene.n_bodies / t, "unit": "sphere-steps/s (forward)", "cores": 1, "kind": "port",
            "sample": "oracle Physics::step (forward) on %d of the %d worlds, mean %.3f s, times %d: %.1f s per "
                      "batch step" % (sample, scene.n_worlds, float(np.mean(ts)), scene.n_worlds, t)}


def max_over_ranks(value, dist, device):
    """The largest `value` over all ranks (the job's time is its slowest
    rank's); `dist` is torch.distributed or None for one process."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(bodies_per_rank, steps, world_size, total_ms):
    """Whole-job sphere-steps/s: every rank steps its own world of
    `bodies_per_rank` bodies `steps` times; the job takes `total_ms`."""
    return world_size * bodies_per_rank * steps / (total_ms / 1e3)


def run_section(args):
    """--section general|batched: one workload alone on one GPU (the launch
    lists and kernel captures under profiles/ are taken of this): `warmup`
    steps, `steps` steps with per-phase CUDA events captured into the step
    graph, then `steps` steps timed with CUDA events, L2 flushed before each;
    one JSON line."""
    import torch
    from blobs_gb300 import native, scenes
    scene = {"general": lambda: scenes.jointed_bodies(),
             "batched": lambda: scenes.uneven_batch(),
             "dense": lambda: scenes.dense_spheres(n=args.n, packing=0.8)}[args.section]()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    w = native.World(scene, device=0)
    w.set_stream(stream.cuda_stream)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    for _ in range(args.warmup):
        w.step(scene.dt)
    w.set_timing(True)
    w.step(scene.dt)  # captures the instrumented graph
    w.phase_times()
    phase = {}
    for _ in range(args.steps):
        flush.zero_()
        w.step(scene.dt)
        for k, (ms, _n) in w.phase_times().items():
            phase[k] = phase.get(k, 0.0) + ms
    w.set_timing(False)
    ms = 0.0
    for _ in range(args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        w.step(scene.dt)
        e1.record(stream)
        torch.cuda.synchronize()
        ms += e0.elapsed_time(e1)
    contacts_last = w.contact_count()[1]
    deferred_last = w.deferred_count()[1] if scene.single_collider() else None
    w.close()
    print(json.dumps({"section": args.section, "bodies": scene.n_bodies, "colliders": scene.n_colliders,
                      "worlds": scene.n_worlds, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": ms / args.steps, "contacts_last_substep": contacts_last,
                      "deferred_bodies_last_substep": deferred_last,
                      "phase_us_per_substep": {k: 1e3 * v / args.steps / scene.substeps for k, v in phase.items()}}),
          flush=True)


def run_reference(args):
    """--impl reference: the reference algorithm's CPU implementation (the
    oracle port; the Rust crate cannot be built here), rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import numpy as np
    from blobs_gb300 import scenes
    from oracle import oracle
    # bounded samples: the whole --steps K run stays within a few minutes
    sizes = [2048, 4096, 8192, 16384] if args.steps <= 30 else [2048, 4096, 8192]
    ns, ts = [], []
    for i in range(args.warmup + args.steps):
        n = sizes[i % len(sizes)]
        s = scenes.dense_spheres(seed=2, n=n)
        w = oracle.OracleWorld(s, 32, maintain_spatial_hash=True)
        w.time_steps(s.dt, 1)
        t = w.time_steps(s.dt, 1)
        if i >= args.warmup:
            ns.append(n)
            ts.append(t)
    A = np.array([[n * n, n] for n in ns], float)
    coef, *_ = np.linalg.lstsq(A, np.array(ts), rcond=None)
    N = args.n
    t_target = float(coef[0] * N * N + coef[1] * N)
    value = N / t_target
    line = {
        "impl": "reference", "metric": "sphere-steps/s @1M", "value": value, "unit": "sphere-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_target * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded dense_spheres generator)",
        "config": {"workload": "1M spheres, r~U[0.05,0.15], 40% packing, dt=1/120, 8 substeps (extrapolated from "
                               "samples)", "bodies": N},
        "cpu_baseline": {"value": value, "unit": "sphere-steps/s", "cores": 1, "kind": "port",
                         "sample": "one oracle step per timed iteration on %s-sphere worlds of the same density, "
                                   "fit t = a N^2 + b N, extrapolated to N=%d" % ("/".join(map(str, sizes)), N)},
        "e2e": {"value": value, "unit": "sphere-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def batched_comparison(dev, steps=100, sample=1024, seed=4):
    """4,096 uneven worlds stepped as one batch (a 100-step rollout captured
    in one CUDA graph) against the per-world form (each world its own device
    world and its own 100-step rollout launch), timed on `sample` evenly
    spaced worlds -- each created, captured, timed and closed in turn -- and
    scaled to all 4,096 by body count."""
    import numpy as np
    import torch
    from blobs_gb300 import native, scenes
    scene = scenes.uneven_batch(seed=seed, steps=steps)
    dt = scene.dt
    stream = torch.cuda.current_stream(dev)
    w = native.World(scene, device=dev.index)
    w.set_stream(stream.cuda_stream)
    # the cell edge picked by timing, as for the headline world (reloads the scene)
    cell_scale = w.autotune(scene, dt, trial_steps=3)
    for _ in range(3):
        w.step(dt)
    w.rollout(dt, steps)  # capture
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    w.rollout(dt, steps)
    e1.record(stream)
    torch.cuda.synchronize()
    batched_ms = e0.elapsed_time(e1)
    w.sync()
    w.close()
    idx = np.unique(np.linspace(0, scene.n_worlds - 1, sample).astype(int))
    sample_ms, bodies = 0.0, 0
    for i in idx:
        sub = scenes.unpack_world(scene, int(i))
        ww = native.World(sub, device=dev.index)
        ww.set_stream(stream.cuda_stream)
        for _ in range(3):
            ww.step(dt)
        ww.rollout(dt, steps)  # capture
        torch.cuda.synchronize()
        e0.record(stream)
        ww.rollout(dt, steps)
        e1.record(stream)
        torch.cuda.synchronize()
        sample_ms += e0.elapsed_time(e1)
        bodies += sub.n_bodies
        ww.close()
    per_world_ms = sample_ms * scene.n_bodies / bodies
    peak, peak_kind = peak_hbm()
    per_body_substep = BYTES_PER_BODY_SUBSTEP + BYTES_PER_SPRING_SUBSTEP * scene.n_springs / scene.n_bodies
    achieved = per_body_substep * scene.substeps * scene.n_bodies * steps / (batched_ms / 1e3) / 1e9
    return {"worlds": scene.n_worlds, "bodies": scene.n_bodies, "springs": scene.n_springs, "steps": steps,
            "cell_scale": cell_scale, "batched_ms": batched_ms, "per_world_ms_est": per_world_ms, "speedup": per_world_ms / batched_ms,
            "batched_sphere_steps_per_s": scene.n_bodies * steps / (batched_ms / 1e3),
            "sample": "%d evenly spaced worlds (%d bodies), one rollout launch per world, scaled by body count"
                      % (len(idx), bodies),
            "roofline": {"bound": "hbm", "alg_bytes_per_body_substep": per_body_substep, "achieved": achieved,
                         "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak},
            "cpu_baseline": cpu_batched(scene)}


def _rollout_ms(w, scene, stream, flush):
    """Every step of the scene's rollout from its loaded state, each between
    its own CUDA-event pair, L2 flushed before each (outside the events)."""
    import numpy as np
    import torch
    n = scene.n_steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
    for e0, e1 in ev:
        flush.zero_()
        e0.record(stream)
        w.step(scene.dt)
        e1.record(stream)
    torch.cuda.synchronize()
    return np.array([e0.elapsed_time(e1) for e0, e1 in ev])


def general_comparison(dev, seed=3):
    """The general path: 200,000 bodies with 1-4 sphere colliders each,
    50,000 fixed joints (4 iterations), 100,000 damped springs, box
    1500 x 1500, dt = 1/120: device time of every step of its 500-step
    rollout from t = 0, on the world's stream."""
    import torch
    from blobs_gb300 import native, scenes
    scene = scenes.jointed_bodies(seed=seed)
    stream = torch.cuda.current_stream(dev)
    w = native.World(scene, device=dev.index)
    w.set_stream(stream.cuda_stream)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    k0 = w.kernel_launches()
    ms = _rollout_ms(w, scene, stream, flush)
    launches = (w.kernel_launches() - k0) / scene.n_steps
    w.close()
    return {"bodies": scene.n_bodies, "colliders": scene.n_colliders, "joints": scene.n_joints,
            "springs": scene.n_springs, "steps": scene.n_steps, "ms_per_step": float(ms.mean()),
            "ms_per_step_first_100": float(ms[:100].mean()), "ms_per_step_last_100": float(ms[-100:].mean()),
            "body_steps_per_s": scene.n_bodies * scene.n_steps / (ms.sum() / 1e3),
            "kernel_launches_per_step": launches, "cpu_baseline": cpu_general()}


def literal_box_comparison(dev, seed=2):
    """The 1,000,000-sphere workload in the literal 2000 x 2000 walled box
    (0.85% packing instead of 40%): device time of every step of its
    1,000-step rollout from t = 0, at the default cell edge and at the edge
    the autotuner picks from the first steps.  Gravity piles the bottom
    bodies on the floor during the rollout, so the sparse start and the
    later pile want different cells."""
    import torch
    from blobs_gb300 import native, scenes
    scene = scenes.dense_spheres(seed=seed, n=1_000_000, literal_box=True)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    runs = {}
    for tuned in (False, True):
        w = native.World(scene, device=dev.index)
        w.set_stream(stream.cuda_stream)
        cell_scale = w.autotune(scene, scene.dt, trial_steps=3) if tuned else 1.0
        ms = _rollout_ms(w, scene, stream, flush)
        contacts_total, contacts_last = w.contact_count()
        deferred_last = w.deferred_count()[1]
        w.close()
        runs[tuned] = {"cell_scale": cell_scale, "ms_per_step": float(ms.mean()),
                       "ms_per_step_first_100": float(ms[:100].mean()),
                       "ms_per_step_last_100": float(ms[-100:].mean()),
                       "sphere_steps_per_s": scene.n_bodies * scene.n_steps / (ms.sum() / 1e3),
                       "contacts_last_substep": contacts_last, "deferred_bodies_last_substep": deferred_last}
    out = {"bodies": scene.n_bodies, "box": float(scene.world_box[0, 2] - scene.world_box[0, 0]),
           "steps": scene.n_steps}
    out.update(runs[False])
    out["autotuned_at_start"] = runs[True]
    return out


def sparse_comparison(dev, seed=1):
    """The 1,000-sphere walled world (600 steps at dt = 1/60) in full: the
    GPU rollout (one step call per step, one CUDA-event pair around all 600)
    against the oracle's single-threaded run of the same 600 steps, with the
    two final states compared bit for bit."""
    import numpy as np
    import torch
    from blobs_gb300 import native, scenes
    from oracle import oracle
    scene = scenes.sparse_spheres(seed=seed)
    stream = torch.cuda.current_stream(dev)
    w = native.World(scene, device=dev.index)
    w.set_stream(stream.cuda_stream)
    w.rollout(scene.dt, scene.n_steps)  # capture the graphs
    w.load(scene)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(scene.n_steps):
        w.step(scene.dt)
    e1.record(stream)
    torch.cuda.synchronize()
    gpu_ms = e0.elapsed_time(e1)
    got = w.read_bodies()
    w.close()
    o = oracle.OracleWorld(scene, 32, maintain_spatial_hash=True)
    cpu_s = o.time_steps(scene.dt, scene.n_steps)
    want = o.bodies()
    exact = all(np.array_equal(got[k].astype(np.float64), want[k]) for k in ("pos", "pos_old", "vel"))
    return {"bodies": scene.n_bodies, "steps": scene.n_steps, "gpu_ms": gpu_ms,
            "gpu_ms_per_step": gpu_ms / scene.n_steps,
            "gpu_sphere_steps_per_s": scene.n_bodies * scene.n_steps / (gpu_ms / 1e3),
            "cpu_baseline": {"value": scene.n_bodies * scene.n_steps / cpu_s, "unit": "sphere-steps/s", "cores": 1,
                             "kind": "port", "seconds": cpu_s,
                             "sample": "the full 600-step run of the oracle, single-threaded"},
            "speedup": cpu_s * 1e3 / gpu_ms, "final_state_bit_exact": exact}


def events_comparison(dev, settle=200, steps=5, seed=2):
    """The headline world with the CollisionEvent stream on (physics.rs:304-311:
    one event per contact per substep): `settle` steps from t = 0 without
    events, one untimed step with them (the step graphs are captured again),
    then `steps` steps with them -- each step between its own
    CUDA-event pair (L2 flushed before it), its events drained to the host
    and put in the reference's order after it (host time, outside the
    events) -- against the same steps with the stream off."""
    import numpy as np
    import torch
    from blobs_gb300 import native, scenes
    scene = scenes.dense_spheres(seed=seed)
    stream = torch.cuda.current_stream(dev)
    w = native.World(scene, device=dev.index)
    w.set_stream(stream.cuda_stream)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    out = {}
    for on in (False, True):
        w.load(scene)
        for _ in range(settle):
            w.step(scene.dt)
        if on:
            w.set_events(True, capacity=12_000_000)
            w.step(scene.dt)  # the step graphs are captured again with the stream on (untimed)
            w.drain_events()
        else:
            w.step(scene.dt)
        ms, drain_s, n_events = [], [], 0
        for _ in range(steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            w.step(scene.dt)
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
            if on:
                t0 = time.perf_counter()
                n_events += len(w.drain_events()[0])
                drain_s.append(time.perf_counter() - t0)
        if on:
            w.set_events(False)
            out["events_on"] = {"ms_per_step": float(np.mean(ms)), "events_per_step": n_events / steps,
                                "drain_ms_per_step": 1e3 * float(np.mean(drain_s))}
        else:
            out["events_off"] = {"ms_per_step": float(np.mean(ms))}
    w.close()
    out.update({"bodies": scene.n_bodies, "steps": "%d-%d of the rollout" % (settle + 1, settle + steps),
                "note": "device time per step with the stream on (the contact kernels append one 32-byte record "
                        "per contact) and off; the drain copies the step's events to the host and sorts them "
                        "into the reference's order"})
    return out


def adjoint_comparison(dev, steps=120, every=16, seed=5, finite_steps=32):
    """256 worlds x 2,048 spheres with 1,024 springs each: a 120-step forward
    pass (one CUDA-graph rollout) against the same rollout recorded with a
    checkpoint every 16 steps plus the backward pass (recompute each
    segment, then the adjoint substeps in reverse).  Every timed leg starts
    from the scene's initial state (the world is reloaded before it) and
    covers steps 0-119; each leg runs once untimed first (graph capture).
    The same legs are timed over the first `finite_steps` steps, a horizon
    whose gradients stay finite in f32."""
    import numpy as np
    import torch
    from blobs_gb300 import native, scenes
    scene, marked, targets = scenes.gradient_batch(seed=seed, steps=steps)
    dt = scene.dt
    stream = torch.cuda.current_stream(dev)
    w = native.World(scene, device=dev.index)
    w.set_stream(stream.cuda_stream)
    M = sum(len(m) for m in marked)
    idx = np.concatenate([int(scene.world_body_offsets[i]) + m for i, m in enumerate(marked)])
    tgt = np.concatenate(targets).astype(np.float64)

    def dl_dx():
        pos = w.read_bodies()["pos"].astype(np.float64)
        g = np.zeros((scene.n_bodies, 2), np.float32)
        g[idx] = 2.0 * (pos[idx] - tgt) / M
        return g

    def legs(n):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        out = {}
        for timed in (False, True):
            w.load(scene)
            torch.cuda.synchronize()
            e0.record(stream)
            w.rollout(dt, n)
            e1.record(stream)
            torch.cuda.synchronize()
            fwd = e0.elapsed_time(e1)
            w.load(scene)
            torch.cuda.synchronize()
            e0.record(stream)
            w.rollout_record(dt, n, every)
            e1.record(stream)
            torch.cuda.synchronize()
            rec = e0.elapsed_time(e1)
            g = dl_dx()
            torch.cuda.synchronize()
            e0.record(stream)
            gv, gk = w.backward(g, scene.n_springs)
            e1.record(stream)
            torch.cuda.synchronize()
            bwd = e0.elapsed_time(e1)
            if timed:
                out = {"steps": n, "fwd_ms": fwd, "fwd_record_ms": rec, "bwd_ms": bwd,
                       "fwd_bwd_over_fwd": (rec + bwd) / fwd,
                       "gradients_finite": bool(np.all(np.isfinite(gv)) and np.all(np.isfinite(gk))),
                       "max_abs_dl_dv0": float(np.nanmax(np.abs(gv)))}
        return out

    full = legs(steps)
    short = legs(finite_steps)
    w.close()
    cpu = cpu_gradient_batch(scene)
    return {"worlds": scene.n_worlds, "bodies": scene.n_bodies, "springs": scene.n_springs, "steps": steps,
            "checkpoint_every": every, "fwd_ms": full["fwd_ms"], "fwd_record_ms": full["fwd_record_ms"],
            "bwd_ms": full["bwd_ms"], "fwd_bwd_over_fwd": full["fwd_bwd_over_fwd"],
            "gradients_finite": full["gradients_finite"],
            "window": "every leg from the scene's initial state (reloaded before it): steps 0-%d" % (steps - 1),
            "finite_horizon": short, "cpu_baseline": cpu,
            "note": "the derivative of this contact dynamics grows by orders of magnitude every few steps "
                    "(max |dL/dv0| of one world: 4e-2 at step 10, 1e1 at 15, 1e12 at 40, 1e84 at 120, f64), so "
                    "the 120-step gradients overflow f32; finite_horizon times the same legs over the first "
                    "%d steps, where they are finite" % finite_steps}


def timed_positions(n_steps, warmup, steps):
    """The K timed steps: evenly spaced over steps W .. n_steps-1 of the
    rollout from t = 0 (every other step runs too, untimed)."""
    span = n_steps - warmup
    if steps > span:
        raise SystemExit("--steps %d exceeds the %d steps after the warm-up" % (steps, span))
    return [warmup + (i * span) // steps for i in range(steps)]


def run_ours(args):
    import numpy as np
    import torch
    from blobs_gb300 import native, scenes

    world_size = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world_size > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)

    scene = scenes.dense_spheres(seed=2 + rank, n=args.n)
    dt = scene.dt
    n_steps = scene.n_steps
    world = native.World(scene, device=local_rank)
    stream = torch.cuda.Stream(dev)          # graphs cannot be captured on the legacy default stream
    torch.cuda.set_stream(stream)
    world.set_stream(stream.cuda_stream)
    # the broadphase cell edge is picked by timing (results do not depend on it);
    # the world is reloaded with the scene's initial state
    cell_scale = world.autotune(scene, dt, trial_steps=3)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MiB > 126 MB L2
    timed = timed_positions(n_steps, args.warmup, args.steps)
    timed_set = set(timed)
    readouts = (1, 200, 500, n_steps)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # -- timed region: the whole rollout from t = 0, every step between its own
    # CUDA-event pair, L2 flushed before each; the K steps at `timed` make `value`
    world.load(scene)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(n_steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(n_steps)]
    counts = {}
    launches = 0
    barrier()
    clocks = Clocks(local_rank)
    clocks.start()
    for i in range(n_steps):
        flush.zero_()
        k0 = world.kernel_launches()
        starts[i].record(stream)
        world.step(dt)
        ends[i].record(stream)
        if i in timed_set:
            launches += world.kernel_launches() - k0
        if i + 1 in readouts:  # synchronising reads, outside the events
            counts[i + 1] = (world.contact_count()[1], world.deferred_count()[1])
    barrier()
    clk = clocks.stop()
    ms = np.array([s_.elapsed_time(e_) for s_, e_ in zip(starts, ends)])
    total_ms = max_over_ranks(float(ms[timed].sum()), dist, dev)
    value = job_throughput(scene.n_bodies, args.steps, world_size, total_ms)
    rollout_ms = max_over_ranks(float(ms.sum()), dist, dev)
    contacts_last = counts[n_steps][0]

    def replay(mode):
        """The same rollout again with per-phase events (mode "all") or
        events around the contact kernel alone ("contact"), summed over the
        timed steps."""
        world.set_timing(True, contact_only=(mode == "contact"))
        world.load(scene)
        world.phase_times()
        acc = {p_: [0.0, 0] for p_ in native.World.PHASES}
        for i in range(n_steps):
            if i in timed_set:
                flush.zero_()
            world.step(dt)
            pt = world.phase_times()  # synchronising; clears the step's marks
            if i in timed_set:
                for p_, (t_, n_) in pt.items():
                    acc[p_][0] += t_
                    acc[p_][1] += n_
        world.set_timing(False)
        return acc

    phase = replay("all")
    contact = replay("contact")["contact"]
    dom_ms = contact[0] / max(1, contact[1])
    peak, peak_kind = peak_hbm()
    alg_bytes = BYTES_CONTACT_PER_BODY * scene.n_bodies
    achieved = alg_bytes / (dom_ms / 1e3) / 1e9

    # -- end to end through the C ABI with pinned host buffers, same steps ----
    n = scene.n_bodies
    h_pos = torch.empty((n, 2), dtype=torch.float32, pin_memory=True).numpy()
    h_old = torch.empty((n, 2), dtype=torch.float32, pin_memory=True).numpy()
    h_vel = torch.empty((n, 2), dtype=torch.float32, pin_memory=True).numpy()
    world.load(scene)
    e2e_s = []
    for i in range(n_steps):
        if i not in timed_set:
            world.step(dt)
            continue
        world.read_bodies_into(h_pos, h_old, h_vel)  # the host copy of the current state (untimed)
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        world.write_bodies(h_pos, h_old)
        world.step(dt)
        world.read_bodies_into(h_pos, h_old, h_vel)   # synchronising
        e2e_s.append(time.perf_counter() - t0)
    e2e_value = job_throughput(n, args.steps, world_size, 1e3 * max_over_ranks(sum(e2e_s), dist, dev))
    world.sync()

    whole_achieved = BYTES_PER_BODY_SUBSTEP * scene.substeps * value / 1e9 / world_size
    line = {
        "metric": "sphere-steps/s @1M", "value": value, "unit": "sphere-steps/s", "n_gpus": world_size,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded dense_spheres generator: uniform positions with overlaps, N(0,0.5) velocities)",
        "config": {"workload": "1M spheres, r~U[0.05,0.15], 40%% packing (side %.1f, walled), g=(0,-9.81), "
                               "dt=1/120, 8 substeps/step, 1,000-step rollout" % (float(scene.world_box[0, 2] * 2)),
                   "bodies": scene.n_bodies, "substeps": scene.substeps, "parallelism": "replicas" if world_size > 1
                   else "single", "l2": "flushed (256 MiB write) before every timed step",
                   "contacts_last_substep": contacts_last, "cell_scale": cell_scale,
                   "window": "the %d-step rollout from t=0 is run in full; the %d timed steps are evenly spaced over "
                             "steps %d-%d (%s); the phase-timing and end-to-end legs reload the scene and time the "
                             "same steps" % (n_steps, args.steps, args.warmup, n_steps - 1,
                                             ",".join(map(str, timed)))},
        "rollout": {"steps": n_steps, "ms_per_step": rollout_ms / n_steps,
                    "value": job_throughput(scene.n_bodies, n_steps, world_size, rollout_ms),
                    "ms_per_step_first_100": float(ms[:100].mean()), "ms_per_step_last_100": float(ms[-100:].mean()),
                    "max_step_ms": float(ms.max()),
                    "contacts_per_substep_after": {str(k): v[0] for k, v in counts.items()},
                    "deferred_bodies_per_substep_after": {str(k): v[1] for k, v in counts.items()},
                    "note": "every step of the configuration's 1,000-step rollout from t=0, each between its own "
                            "CUDA-event pair, L2 flushed before each (outside the events); the counts are of the "
                            "last substep after 1, 200, 500 and 1,000 steps"},
        "roofline": {"bound": "hbm", "kernel": "k_step_single (contact + integration)", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                     "alg_bytes_per_launch": alg_bytes, "avg_launch_ms": dom_ms,
                     "timing": "CUDA events around the contact kernel alone, captured into the step graph, over "
                               "the timed steps",
                     "traffic": profile_traffic("k_step_single_1M.md"),
                     "step_alg_GBps": whole_achieved, "step_frac": whole_achieved / peak},
        "phases_ms_per_step": {p_: phase[p_][0] / args.steps for p_ in phase},
        "e2e": {"value": e2e_value, "unit": "sphere-steps/s", "h2d_bytes_per_step": 16 * n,
                "d2h_bytes_per_step": 24 * n},
        "gpu_launches": launches,
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(target_n=scene.n_bodies)
    world.close()
    if rank == 0 and not args.no_sparse:
        line["sparse_1k"] = sparse_comparison(dev)
    if rank == 0 and not args.no_batched:
        line["batched"] = batched_comparison(dev)
    if rank == 0 and not args.no_adjoint:
        line["adjoint"] = adjoint_comparison(dev)
    if rank == 0 and not args.no_events:
        line["events"] = events_comparison(dev)
    if rank == 0 and not args.no_general:
        line["general"] = general_comparison(dev)
    if rank == 0 and not args.no_literal:
        line["literal_box"] = literal_box_comparison(dev)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1_000_000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-general", action="store_true")
    ap.add_argument("--no-literal", action="store_true", help="skip the 2000 x 2000 literal-box run")
    ap.add_argument("--no-sparse", action="store_true", help="skip the 1,000-sphere full-run comparison")
    ap.add_argument("--no-events", action="store_true", help="skip the collision-event stream comparison")
    ap.add_argument("--section", choices=["general", "batched", "dense"], default=None,
                    help="run one secondary workload alone (profiling driver), print its phase times; dense: the "
                         "1M-sphere world at 80%% packing, the density of the rollout's settled pile")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.section:
        run_section(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
