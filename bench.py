#!/usr/bin/env python
"""Throughput of the PyRDSim simulation step on GB300 (particle-steps/s).

Workload (default): the 2D active wall fluid -- N = 65,536 particles at
density 0.4, periodic in x, reflecting in y, WCA between inactive particles,
LJ (cut 2.5) between active ones, a 9-3 wall attracting active particles to
y = 0, activation at rate 0.1 and deactivation at rate 1.0 per active
neighbour within 1.5.  dt = 1e-4, forces float32, positions 64-bit fixed
point, counter-based Philox noise.  Synthetic, seeded input.

One bench step = one segment of 1,000 integration steps (the workload's
20,000 steps are 20 bench steps).  The state (a few MB) is L2-resident
between integration steps by construction; L2 is flushed (256 MB write)
between timed segments.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun each rank runs an independent replica (replicas only: the
single-system path has no data-path exchange), and rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s on 1 GB300 (active wall fluid, N=65,536)"
UNIT = "particle-steps/s"
SEGMENT = 1000
ALG_BYTES = 40  # per particle-step: 16 B read x, 16 B write x, 4 B type read, 4 B type write
# Steps between the engine's Verlet-list rebuilds in the timed runs (the deck
# of the workload keeps the reference's default neighbor_list_update_frequency
# of 10; the engine's skin grows with the period and its displacement check
# keeps every pair in range listed, so the dynamics are the same).
LIST_PERIOD = 20


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=65536)
    p.add_argument("--segment", type=int, default=SEGMENT)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-ensemble", action="store_true")
    p.add_argument("--no-adjoint", action="store_true")
    p.add_argument("--no-precision", action="store_true")
    p.add_argument("--no-sweep", action="store_true")
    return p.parse_args()


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if _has_cuda() else "gloo")
    return rank, ws, local


def _has_cuda():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, ws):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if _has_cuda() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except Exception:
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def traffic_per_launch(n, steps=1, period=False):
    """dram bytes per launch of the dominant kernel (k_period: ``steps``
    integration steps per launch; k_force_l: one) from the committed ncu
    summary, per particle and step, or None."""
    name = "k_period_active_wall_fluid.md" if period else "k_force_l_active_wall_fluid.md"
    key = "traffic_bytes_per_particle_step:" if period else "traffic_bytes_per_particle:"
    try:
        with open(os.path.join(ROOT, "profiles", name)) as f:
            for line in f:
                if line.startswith(key):
                    return float(line.split(":")[1]) * n * steps
    except Exception:
        pass
    return None


def dominant_kernel(eng, sd):
    """(kernel name, integration steps per launch) of the drift work: the
    period kernel runs a whole list period per launch."""
    info = eng.info()
    if info["period_kernel"]:
        return "k_period<2,2>", int(info["list_period"])
    return "k_force_l<2,2>", 1


def cpu_baseline(workload, n_gpu_state=None):
    """Reference (compiled PyRDSim) on a bounded sample, one core."""
    from oracle import ref_bench
    kind = "reference" if ref_bench.reference_available() else "port"
    n, steps = (4096, 20) if kind == "reference" else (65536, 20)
    secs = ref_bench.run_sample(kind, workload, n, steps, 5)
    return {
        "value": n * steps / secs, "unit": UNIT, "cores": 1, "kind": kind,
        "sample": (f"{workload} shape at N={n} (density 0.4, tanh wall in place of the "
                   f"9-3 wall), {steps} integration steps incl. {steps // 10} neighbour "
                   f"rebuilds, set-up excluded, {secs:.2f} s") if kind == "reference" else
                  (f"float64 oracle port, {workload} N={n}, {steps} steps, {secs:.2f} s"),
    }


def _port_worker(a):
    from oracle import ref_bench
    workload, n, steps, seed = a
    return ref_bench.run_sample("port", workload, n, steps, seed)


def cpu_baseline_port_all_cores(n=65536, steps=5):
    """Secondary CPU baseline: the float64 C++ restatement of the step (cell
    lists, O(N)) at the full N, one independent replica per host core
    (spawned processes), throughput summed over the replicas."""
    import multiprocessing as mp
    procs = max(1, os.cpu_count() or 1)
    with mp.get_context("spawn").Pool(procs) as pool:
        pool.map(_port_worker, [("active_wall_fluid", 4096, 1, p) for p in range(procs)])
        t0 = time.perf_counter()
        secs = pool.map(_port_worker, [("active_wall_fluid", n, steps, 50 + p)
                                       for p in range(procs)])
        wall = time.perf_counter() - t0
    return {"value": procs * n * steps / max(secs), "unit": UNIT, "cores": procs, "kind": "port",
            "sample": f"float64 C++ restatement (cell lists), active wall fluid at N={n} "
                      f"(tanh wall), {procs} replicas x {steps} steps each, one per core, "
                      f"slowest replica {max(secs):.2f} s (wall {wall:.2f} s)"}


def fp64_drift(sd, x, types, device):
    """Plain PyTorch float64 drift of one system at positions x: the pair laws
    (pyrdsim.pyx:1068-1130) over every pair of different molecules within
    each law's cutoff (the (small, large) type pair as listed; minimum image
    in periodic dimensions), the walls (pyrdsim.pyx:1132-1145; the 9-3 wall
    cut at rc) and the bonds (pyrdsim.pyx:2037-2047).  Dense in chunks of
    rows; angle terms are not covered."""
    import numpy as np
    import torch
    m = sd.model
    D, N = m.N_dim, sd.n_particles
    f64 = dict(dtype=torch.float64, device=device)
    X = torch.tensor(np.asarray(x)[:, :D], **f64)
    T = torch.tensor(np.asarray(types), dtype=torch.long, device=device)
    mol = torch.tensor(sd.molecule_ids[:, 0], dtype=torch.long, device=device)
    L = torch.tensor(np.asarray(m.L, dtype=float)[:D], **f64)
    per = torch.tensor(np.asarray(m.periodic, dtype=float)[:D] > 0, device=device)
    laws = [sd.inter[q] for q in range(sd.struct.n_interactions)]
    pair_laws = [w for w in laws if 1 <= w.law <= 5 and w.type_a <= w.type_b]
    walls = [w for w in laws if w.law in (6, 7)]

    def law_f(w, r):
        if w.law == 1:
            s = (w.r0 / r) ** w.n
            return -2.0 * w.n * w.u0 / r * s * (s - 1.0)
        if w.law == 2:
            return w.u0 * (1.0 - torch.tanh((r - w.r0) / w.a) ** 2) / (2.0 * w.a)
        if w.law == 3:
            return -w.u0 * (1.0 + w.r0 / r) * torch.exp(-r / w.r0) / (r * w.r0)
        if w.law == 4:
            return w.u0 * r
        return torch.where(r < w.r0 - w.dr, torch.zeros_like(r), torch.full_like(r, w.u0 / w.dr))

    a = torch.zeros_like(X)
    ch = max(1, (1 << 27) // N)
    for i0 in range(0, N, ch):
        i1 = min(N, i0 + ch)
        d = X[None, :, :] - X[i0:i1, None, :]
        d = torch.where(per, d - L * torch.round(d / L), d)
        r = torch.sqrt((d * d).sum(-1))
        other = (mol[i0:i1, None] != mol[None, :]) & (r > 0)
        lo = torch.minimum(T[i0:i1, None], T[None, :])
        hi = torch.maximum(T[i0:i1, None], T[None, :])
        rs = torch.where(other, r, torch.ones_like(r))
        fr = torch.zeros_like(r)
        for w in pair_laws:
            rc = w.r0 if w.law == 5 else w.rc
            mask = other & (lo == w.type_a) & (hi == w.type_b) & (r <= rc)
            fr = fr + torch.where(mask, law_f(w, rs) / rs, torch.zeros_like(r))
        a[i0:i1] += (fr[..., None] * d).sum(1)
        del d, r, other, lo, hi, rs, fr
    for w in walls:
        sel = T == w.type_a
        y = X[:, w.type_b]
        if w.law == 6:
            f = w.u0 * (1.0 - torch.tanh((y - w.r0) / w.a) ** 2) / (2.0 * w.a)
        else:
            sr = w.r0 / y
            f = torch.where(y <= w.rc, w.u0 / y * (-1.2 * sr ** 9 + 3.0 * sr ** 3), torch.zeros_like(y))
        a[:, w.type_b] -= torch.where(sel, f, torch.zeros_like(f))
    # bonds of every molecule
    i1s, i2s, ks, r0s = [], [], [], []
    tmpl = {sd.tmpl[q].molecule_id: sd.tmpl[q] for q in range(sd.struct.n_templates)}
    for first in sd.first_index:
        tp = tmpl.get(int(sd.molecule_ids[first, 2]))
        if tp is None:
            continue
        for e in range(tp.first_term, tp.first_term + tp.n_terms):
            tm = sd.terms[e]
            if tm.kind == 1:
                i1s.append(first + tm.i)
                i2s.append(first + tm.j)
                ks.append(tm.k0)
                r0s.append(tm.p0)
    if i1s:
        i1 = torch.tensor(i1s, device=device)
        i2 = torch.tensor(i2s, device=device)
        v = X[i2] - X[i1]
        v = torch.where(per, v - L * torch.round(v / L), v)
        dist = torch.sqrt((v * v).sum(-1))
        f = torch.tensor(ks, **f64) * (dist - torch.tensor(r0s, **f64))
        g = (f / dist)[:, None] * v
        a.index_add_(0, i1, g)
        a.index_add_(0, i2, -g)
    return a.cpu().numpy()


def force_error(eng, sd, device):
    """Drift of the GPU engine (float32 pair and bonded forces) against the
    float64 PyTorch drift at the same state, right after a rebuild."""
    import numpy as np
    x, t = eng.state()
    eng.set_state(x, t)
    x, t = eng.state()
    a, r = eng.drift(), fp64_drift(sd, x, t, device)
    norm = float(np.linalg.norm(a - r) / np.linalg.norm(r))
    mag = np.linalg.norm(r, axis=1)
    floor = float(np.sqrt(np.mean(mag ** 2)))
    per = float((np.linalg.norm(a - r, axis=1) / np.maximum(mag, floor)).max())
    return {"norm": norm, "per_particle_rms_floor": per}


def _events_ms(stream_ptrs, fn):
    """Run fn() between CUDA events recorded on the first and last of the
    engines' streams (fn synchronises each engine it steps); device ms."""
    import torch
    s0 = torch.cuda.ExternalStream(stream_ptrs[0])
    s1 = torch.cuda.ExternalStream(stream_ptrs[-1])
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(s0)
    fn()
    b.record(s1)
    torch.cuda.synchronize()
    return a.elapsed_time(b)


def trajectory_error(sds, local, steps=100, seed=11):
    """Positions after ``steps`` injected-noise steps of the float32 engine
    against the float64 engine (precision="float64", pinned to the oracle at
    1e-12 by the GPU tests) from the same thermalised state; the uniforms are
    1 so that no reaction fires.  Max absolute and relative differences."""
    import numpy as np
    from pyrdsim_gb300.engine import Engine
    f32 = Engine(sds, device=local)
    f32.step(200)
    x0, t0 = f32.state()
    f64 = Engine(sds, device=local, precision="float64")
    f64.set_state(x0, t0)
    f32.set_state(x0, t0)
    n, D = f32.N, f32.D
    rng = np.random.default_rng(seed)
    ones = np.ones((10, n))
    for c in range(steps // 10):
        xi = rng.standard_normal((10, n, D))
        f32.step(10, xi=xi, u1=ones, u2=ones)
        f64.step(10, xi=xi, u1=ones, u2=ones)
    xa, _ = f32.state()
    xb, _ = f64.state()
    d = xa - xb
    off = 0
    for sd in sds:
        m = sd.model
        sl = slice(off, off + sd.n_particles)
        for k in range(D):
            if m.periodic[k] > 0:
                d[sl, k] -= m.L[k] * np.round(d[sl, k] / m.L[k])
        off += sd.n_particles
    f32.close()
    f64.close()
    return {"max_abs": float(np.abs(d).max()),
            "max_rel": float((np.abs(d) / np.maximum(np.abs(xb), 1.0)).max()),
            "steps": steps}


def precision_report(local):
    """For every configuration's shape: the float32 drift against the plain
    PyTorch float64 drift after 200 thermalising steps (the patchy colloids
    start with every bond at rest), and positions after 100 injected-noise
    steps against the float64 engine."""
    from pyrdsim_gb300 import workloads
    from pyrdsim_gb300.engine import Engine
    dev = f"cuda:{local}"
    out = {}
    cases = {
        "cfg1_lj_fluid_n1024": [workloads.lj_fluid(n=1024)],
        "cfg2_active_wall_fluid_n65536": [workloads.active_wall_fluid(n=65536)],
        "cfg3_patchy_colloids_n65536": [workloads.patchy_colloids(n_molecules=16384)],
        "cfg4_ensemble_8_systems": workloads.ensemble(n_systems=8, seed=4),
    }
    for name, sds in cases.items():
        errs = []
        for sd in sds:
            eng = Engine([sd], device=local)
            eng.step(200)
            errs.append(force_error(eng, sd, dev))
            eng.close()
        row = {"force_norm": max(q["norm"] for q in errs),
               "force_per_particle_rms_floor": max(q["per_particle_rms_floor"] for q in errs)}
        try:
            row["positions_after_100_steps"] = trajectory_error(sds, local)
        except Exception as exc:
            row["positions_after_100_steps"] = {"unavailable": str(exc)[:200]}
        out[name] = row
    return out


def ensemble_comparison(local, steps=5000, n_systems=512, f64_sample=64):
    """The 512-system ensemble: batched (all systems in one handle, autotuned
    geometry) against the plain per-system form (one handle per system,
    stepped one system at a time) with the default and with the autotuned
    geometry, all over the configuration's 5,000 steps with Philox noise,
    timed with CUDA events on the engines' streams; and the plain form in
    float64 (the reference's precision) on every (512 / f64_sample)-th
    system, scaled by particles.  Rebuild periods replay as CUDA graphs of
    neighbor_list_update_frequency (10) steps: a graph of 100 steps would
    hold 10 rebuild periods and change nothing but the launch of the graph
    itself (one launch per ten steps here)."""
    from pyrdsim_gb300 import workloads
    from pyrdsim_gb300.engine import Engine
    from pyrdsim_gb300.autotune import autotune
    sds = workloads.ensemble(n_systems=n_systems)
    total = sum(s.n_particles for s in sds)
    tuned = autotune(sds, device=local, steps=100)
    tpp = tuned["threads_per_particle"] or 0
    out = {"n_systems": n_systems, "n_particles": total, "steps": steps, "unit": UNIT,
           "batched_options": tuned,
           "workload": "512 systems, N log-uniform [256, 16384], density U[0.2, 0.7], "
                       "kT U[0.5, 2], LJ or Yukawa, half with two-state reactions"}
    clocks = ClockSampler(local)
    batch = Engine(sds, device=local, skin=tuned["skin"], threads_per_particle=tpp)
    batch.step(100)
    ms = _events_ms([batch.stream()], lambda: batch.step(steps))
    batch.close()
    out["batched"] = total * steps / (ms / 1e3)
    for label, kw in (("plain_per_system", {}),
                      ("plain_per_system_autotuned", {"skin": tuned["skin"],
                                                      "threads_per_particle": tpp})):
        engines = [Engine([s], device=local, **kw) for s in sds]
        for e in engines:
            e.step(20)
        ms = _events_ms([e.stream() for e in engines],
                        lambda: [e.step(steps) for e in engines])
        for e in engines:
            e.close()
        out[label] = total * steps / (ms / 1e3)
    sample = sds[::max(1, n_systems // f64_sample)]
    engines = [Engine([s], device=local, precision="float64") for s in sample]
    for e in engines:
        e.step(20)
    ms = _events_ms([e.stream() for e in engines], lambda: [e.step(steps) for e in engines])
    for e in engines:
        e.close()
    out["plain_per_system_float64"] = sum(s.n_particles for s in sample) * steps / (ms / 1e3)
    out["plain_float64_sample"] = f"{len(sample)} of {n_systems} systems (every " \
                                  f"{max(1, n_systems // f64_sample)}th), {steps} steps"
    out["speedup"] = out["batched"] / out["plain_per_system"]
    out["speedup_vs_autotuned_plain"] = out["batched"] / out["plain_per_system_autotuned"]
    out["speedup_vs_float64_plain"] = out["batched"] / out["plain_per_system_float64"]
    out["clocks"] = clocks.stop()
    try:
        errs = [force_error_of(sd, local) for sd in sds[::64]]
        out["force_err_vs_fp64_batched_geometry"] = {
            "norm": max(q["norm"] for q in errs),
            "per_particle_rms_floor": max(q["per_particle_rms_floor"] for q in errs),
            "systems": len(errs)}
    except Exception as exc:
        out["force_err_vs_fp64_batched_geometry"] = {"unavailable": str(exc)[:200]}
    return out


def force_error_of(sd, local):
    from pyrdsim_gb300.engine import Engine
    eng = Engine([sd], device=local)
    eng.step(200)
    r = force_error(eng, sd, f"cuda:{local}")
    eng.close()
    return r


def lj_fluid_plain_method(local, steps=10000):
    """The 2D LJ fluid (N = 1,024, density 0.5, relaxed uniform start) over
    its stated 10,000 steps with the float64 plain method and with the
    float32 forces; CUDA events on the engine stream."""
    from pyrdsim_gb300 import workloads
    from pyrdsim_gb300.engine import Engine
    sd = workloads.lj_fluid(n=1024)
    out = {"workload": "2D LJ fluid, N=1024, density 0.5, dt=1e-4, relaxed uniform start",
           "steps": steps, "unit": UNIT}
    for prec in ("float64", "float32"):
        eng = Engine([sd], device=local, precision=prec)
        eng.step(100)
        ms = _events_ms([eng.stream()], lambda: eng.step(steps))
        out[prec] = sd.n_particles * steps / (ms / 1e3)
        eng.close()
    return out


def deck_period_value(sd, local, seg, flush, segments=6):
    """Particle-steps/s of the headline loop (CUDA events on the engine
    stream, L2 flushed between segments) with the engine's list period equal
    to the deck's neighbor_list_update_frequency."""
    import torch
    from pyrdsim_gb300.engine import Engine
    eng = Engine([sd], device=local)
    stream = torch.cuda.ExternalStream(eng.stream())
    eng.step(seg)
    ms = 0.0
    for _ in range(segments):
        with torch.cuda.stream(stream):
            flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.step(seg)
        b.record(stream)
        torch.cuda.synchronize()
        ms += a.elapsed_time(b)
    out = {"value": sd.n_particles * seg * segments / (ms / 1e3), "unit": UNIT,
           "list_period": sd.model.neighbor_list_update_frequency, "segments": segments,
           "ms_per_step": ms / segments}
    eng.close()
    return out


def n_sweep(local, sizes=((65536, 1000), (1048576, 200), (4194304, 100))):
    """The active wall fluid at growing N (density 0.4): throughput and the
    drift kernel's average launch span (device timestamps of the timed
    replays) against the measured HBM peak.  At 65,536 particles the state
    (~25 MB) lives in L2; at 4M (~1.5 GB) it cannot."""
    from pyrdsim_gb300 import workloads
    from pyrdsim_gb300.engine import Engine
    import torch
    peak, _ = peaks()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    rows = []
    for n, steps in sizes:
        sd = workloads.active_wall_fluid(n=n)
        eng = Engine([sd], device=local, list_period=LIST_PERIOD)
        eng.set_profiling(False, stamps=True)
        eng.step(steps)
        eng.profile()
        flush.zero_()
        ms = _events_ms([eng.stream()], lambda: eng.step(steps))
        prof = eng.profile()
        span = prof["drift_span"]
        kname, per = dominant_kernel(eng, sd)
        us = 1e3 * span["ms"] / max(1, span["launches"])
        ach = ALG_BYTES * n * per / (us / 1e6) / 1e9
        rows.append({"n_particles": n, "steps": steps,
                     "particle_steps_per_s": n * steps / (ms / 1e3),
                     "us_per_step": 1e3 * ms / steps, "kernel": kname,
                     "steps_per_launch": per,
                     "drift_span_us": us, "drift_achieved_gbs": ach,
                     "drift_frac_of_measured_hbm": ach / peak,
                     "device_bytes": eng.info()["device_bytes"]})
        eng.close()
        del sd
    return rows


def adjoint_timing(local, n=16384, steps=1000, loss_steps=500, every=32, reps=2):
    """Loss and gradients of the reaction-free mixture (LJ + Yukawa, N =
    16,384, density 0.5, 1,000 steps, loss over the last 500 states,
    checkpoints every 32 steps): wall time of the forward and the backward
    call (each returns after synchronising its stream), best of ``reps``."""
    import numpy as np
    import torch
    from pyrdsim_gb300 import workloads
    from pyrdsim_gb300.adjoint import Adjoint
    w = workloads.mixed_lj_yukawa(n=n)
    adj = Adjoint(2, w["L"], w["dt"], w["mobility"], w["types"],
                  workloads.mixed_lj_yukawa_laws(w), loss_steps=loss_steps,
                  checkpoint_every=every, device=local)
    gen = torch.Generator(device=f"cuda:{local}").manual_seed(5)
    xi = torch.randn((steps, n, 2), dtype=torch.float64, device=f"cuda:{local}", generator=gen)
    x0 = torch.tensor(w["x0"], dtype=torch.float64, device=f"cuda:{local}")
    p = workloads.mixed_lj_yukawa_params(w["theta"])
    best_f = best_b = float("inf")
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        loss, _ = adj.forward(x0, p, xi)
        t1 = time.perf_counter()
        gx, gp = adj.backward()
        t2 = time.perf_counter()
        best_f, best_b = min(best_f, t1 - t0), min(best_b, t2 - t1)
    adj.close()
    return {"workload": "2D LJ+Yukawa mixture, N=16384, density 0.5, 1000 steps, loss over the "
                        "last 500 states, checkpoints every 32 steps, float64",
            "forward_ms": 1e3 * best_f, "backward_ms": 1e3 * best_b,
            "particle_steps_per_s_forward": n * steps / best_f,
            "particle_steps_per_s_forward_backward": n * steps / (best_f + best_b),
            "loss": loss, "grad_params_norm": float(np.linalg.norm(gp.numpy())),
            "grad_x0_norm": float(gx.norm())}


def run_ours(args, rank, ws, local):
    import torch
    from pyrdsim_gb300 import workloads
    from pyrdsim_gb300.engine import Engine
    torch.cuda.set_device(local)
    sd = workloads.active_wall_fluid(n=args.n, seed=2 + rank)
    eng = Engine([sd], device=local, list_period=LIST_PERIOD)
    # the drift kernel stamps each CTA's start and end in the timed replays
    eng.set_profiling(False, stamps=True)
    N, seg = sd.n_particles, args.segment
    stream = torch.cuda.ExternalStream(eng.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    x0, t0 = eng.state()
    for _ in range(args.warmup):
        eng.step(seg)
    torch.cuda.synchronize()
    eng.profile()  # reset counters and stamps
    barrier(ws)
    clocks = ClockSampler(local) if rank == 0 else None
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    torch.cuda.synchronize()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        starts[k].record(stream)
        eng.step(seg)
        ends[k].record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    clk = clocks.stop() if clocks else None
    timed = eng.profile()
    seg_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = sum(seg_ms)
    ms_max = max_over_ranks(ms, ws)
    value = ws * N * seg * args.steps / (ms_max / 1e3)
    launches = sum(v["launches"] for k, v in timed.items() if k not in ("hook", "drift_span"))
    span = timed["drift_span"]
    span_us = 1e3 * span["ms"] / max(1, span["launches"])
    peak, peak_kind = peaks()
    kname, per = dominant_kernel(eng, sd)
    achieved = ALG_BYTES * N * per / (span_us / 1e6) / 1e9
    traffic = traffic_per_launch(N, per, per > 1)
    # a short serialised pass (CUDA events around every launch; no graphs)
    # for the per-class split; not the timed pass
    eng.set_profiling(True, stamps=False)
    for k in range(2):
        eng.step(seg)
    torch.cuda.synchronize()
    ser = eng.profile()
    eng.set_profiling(False)
    # end to end through the C ABI with host buffers: state in, segment, state out
    xh = torch.empty((N, 2), dtype=torch.float64, pin_memory=True).numpy()
    th = torch.empty((N,), dtype=torch.int32, pin_memory=True).numpy()
    xh[:] = x0
    th[:] = t0
    xo = torch.empty((N, 2), dtype=torch.float64, pin_memory=True).numpy()
    to = torch.empty((N,), dtype=torch.int32, pin_memory=True).numpy()
    e2e_t = 0.0
    for k in range(args.steps):
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        eng.set_state(xh, th)
        eng.step(seg)
        eng.state(xo, to)
        torch.cuda.synchronize()
        e2e_t += time.perf_counter() - w0
    e2e_t = max_over_ranks(e2e_t, ws)
    e2e = ws * N * seg * args.steps / e2e_t
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 forces, i64 fixed-point x, f64 rates",
        "data": "synthetic (seeded jittered lattice, 50/50 species)",
        "config": {"workload": "active_wall_fluid", "n_particles": N, "density": 0.4,
                   "integration_steps_per_step": seg, "dt": 1e-4,
                   "boundaries": "periodic x, reflecting y", "noise": "Philox4x32-10",
                   "l2": "flushed (256 MB write) between timed steps; state L2-resident "
                         "within a step", "parallelism": f"replicas x{ws}",
                   "neighbor_list_update_frequency": sd.model.neighbor_list_update_frequency,
                   "engine_list_period": LIST_PERIOD},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(N * 2 * 8 + N * 4),
                "d2h_bytes_per_step": int(N * 2 * 8 + N * 4),
                "path": "C ABI: rdsim_set_state (host) + rdsim_step + rdsim_get_state (host)"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "kernel": kname,
                     "integration_steps_per_launch": per,
                     "algorithmic_bytes_per_launch": ALG_BYTES * N * per,
                     "avg_launch_us": span_us, "launches_timed": span["launches"],
                     "timing": "device global-timer stamps in the timed graph replays: last "
                               "CTA end minus first CTA start, averaged over the launches",
                     "peak_source": peak_kind,
                     "drift_share_of_timed": span["ms"] / ms},
        "segment_us_per_step": [round(1e3 * m / seg, 3) for m in seg_ms],
        "kernel_launches": {k: v["launches"] for k, v in timed.items() if k != "drift_span"},
        "serialised_kernel_us": {k: 1e3 * v["ms"] / max(1, v["timed"])
                                 for k, v in ser.items() if k != "drift_span" and v["timed"]},
        "clocks": clk,
        "engine": eng.info(),
    }
    if rank == 0 and ws == 1:
        # the same timed loop with the engine rebuilding at the deck's own
        # neighbor_list_update_frequency (fewer segments)
        try:
            out["value_at_deck_list_period"] = deck_period_value(sd, local, seg, flush)
        except Exception as exc:
            out["value_at_deck_list_period"] = {"unavailable": str(exc)[:200]}
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        try:
            out["cpu_baseline"] = cpu_baseline("active_wall_fluid")
        except Exception as exc:
            out["cpu_baseline"] = {"unavailable": str(exc)[:200]}
        try:
            out["cpu_baseline_all_cores"] = cpu_baseline_port_all_cores()
        except Exception as exc:
            out["cpu_baseline_all_cores"] = {"unavailable": str(exc)[:200]}
        try:
            out["force_err_vs_fp64"] = force_error(eng, sd, f"cuda:{local}")
        except Exception as exc:
            out["force_err_vs_fp64"] = {"unavailable": str(exc)[:200]}
    eng.close()
    extras = [("precision_vs_fp64", args.no_precision, precision_report),
              ("lj_fluid_plain_method", args.no_precision, lj_fluid_plain_method),
              ("ensemble", args.no_ensemble, ensemble_comparison),
              ("n_sweep", args.no_sweep, n_sweep),
              ("adjoint", args.no_adjoint, adjoint_timing)]
    if rank == 0 and ws == 1:
        for key, skip, fn in extras:
            if skip:
                continue
            try:
                out[key] = fn(local)
            except Exception as exc:
                out[key] = {"unavailable": str(exc)[:200]}
    if rank == 0:
        print(json.dumps(out))


def _ref_worker(a):
    from oracle import ref_bench
    kind, workload, n, steps, seed = a
    return ref_bench.run_sample(kind, workload, n, steps, seed)


def run_reference(args, rank, ws):
    if rank != 0:
        return
    import multiprocessing as mp
    from oracle import ref_bench
    kind = "reference" if ref_bench.reference_available() else "port"
    n, steps = (4096, 10) if kind == "reference" else (65536, 5)
    procs = max(1, min(16, os.cpu_count() or 1))
    ctx = mp.get_context("spawn")
    total_ps, total_t = 0.0, 0.0
    with ctx.Pool(procs) as pool:
        for k in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            secs = pool.map(_ref_worker, [(kind, "active_wall_fluid", n, steps, 100 * k + p)
                                          for p in range(procs)])
            if k >= args.warmup:
                total_ps += procs * n * steps
                total_t += max(secs)
    value = total_ps / total_t
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total_t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded jittered lattice, 50/50 species)",
        "config": {"workload": "active_wall_fluid", "n_particles": n, "density": 0.4,
                   "integration_steps_per_step": steps, "dt": 1e-4,
                   "parallelism": f"{procs} independent single-threaded processes"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": kind,
                         "sample": f"{procs} processes x N={n} (tanh wall for the 9-3 wall), "
                                   f"{steps} integration steps each per step, set-up excluded"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def main():
    args = parse()
    rank, ws, local = dist_init()
    if args.impl == "reference":
        run_reference(args, rank, ws)
    else:
        run_ours(args, rank, ws, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
