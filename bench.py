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


def traffic_per_launch(n):
    """dram bytes per k_force_l launch from the committed ncu summary (scaled
    by particles if the capture was a smaller case), or None."""
    path = os.path.join(ROOT, "profiles", "k_force_l_active_wall_fluid.md")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_particle:"):
                    return float(line.split(":")[1]) * n
    except Exception:
        pass
    return None


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


def precision_report(local):
    """Force error against float64 for every configuration's shape after 200
    thermalising steps (the patchy colloids start with every bond at rest,
    where the relative error of near-zero bond forces says nothing), and the
    trajectory error of the reaction-free LJ fluid after 100 steps with the
    same injected normals (float64 PyTorch integration)."""
    import numpy as np
    import torch
    from pyrdsim_gb300 import workloads
    from pyrdsim_gb300.engine import Engine
    dev = f"cuda:{local}"
    out = {}
    cases = {
        "cfg1_lj_fluid_n1024": workloads.lj_fluid(n=1024),
        "cfg3_patchy_colloids_n65536": workloads.patchy_colloids(n_molecules=16384),
        "cfg4_ensemble_8_systems": None,
    }
    for name, sd in cases.items():
        if sd is None:
            errs = []
            for e in workloads.ensemble(n_systems=8, seed=4):
                eng = Engine([e], device=local)
                eng.step(200)
                errs.append(force_error(eng, e, dev))
            out[name] = {"norm": max(q["norm"] for q in errs),
                         "per_particle_rms_floor": max(q["per_particle_rms_floor"] for q in errs)}
        else:
            eng = Engine([sd], device=local)
            eng.step(200)
            out[name] = force_error(eng, sd, dev)
    # trajectory: 100 steps of the LJ fluid, noise injected into both
    sd = workloads.lj_fluid(n=1024)
    eng = Engine([sd], device=local)
    x0, t0 = eng.state()
    rng = np.random.default_rng(11)
    xi = rng.standard_normal((100, sd.n_particles, 2))
    eng.step(100, xi=xi, u1=np.ones((100, sd.n_particles)), u2=np.ones((100, sd.n_particles)))
    xg, _ = eng.state()
    m = sd.model
    L = np.asarray(m.L, dtype=float)[:2]
    D_t = float(m.tau_by_tauD[0])
    x = x0.copy()
    for k in range(100):
        a = fp64_drift(sd, x, t0, dev)
        x = x + m.dt * D_t * a
        x = x + np.sqrt(2.0 * m.dt * D_t) * xi[k]
        x = np.mod(x, L)
    d = xg - x
    d -= L * np.round(d / L)
    out["cfg1_lj_fluid_n1024_positions_after_100_steps"] = {
        "max_abs": float(np.abs(d).max()),
        "max_rel": float((np.abs(d) / np.maximum(np.abs(x), 1.0)).max())}
    return out


def ensemble_comparison(local, steps=100, n_systems=512):
    """Batched ensemble (all systems in one handle, one launch per kernel per
    step) vs the plain per-system form (one handle per system, stepped one
    system at a time), both on the GPU with Philox noise."""
    import torch
    from pyrdsim_gb300 import workloads
    from pyrdsim_gb300.engine import Engine
    from pyrdsim_gb300.autotune import autotune
    sds = workloads.ensemble(n_systems=n_systems)
    total = sum(s.n_particles for s in sds)
    tuned = autotune(sds, device=local, steps=steps)
    batch = Engine(sds, device=local, skin=tuned["skin"],
                   threads_per_particle=tuned["threads_per_particle"] or 0)
    batch.step(steps // 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    batch.step(steps)
    torch.cuda.synchronize()
    t_b = time.perf_counter() - t0
    batch.close()
    engines = [Engine([s], device=local) for s in sds]
    for e in engines:
        e.step(steps // 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for e in engines:
        e.step(steps)
    torch.cuda.synchronize()
    t_p = time.perf_counter() - t0
    for e in engines:
        e.close()
    b = total * steps / t_b
    p = total * steps / t_p
    return {"n_systems": n_systems, "n_particles": total, "steps": steps,
            "batched": b, "plain_per_system": p, "speedup": b / p, "unit": UNIT,
            "batched_options": tuned,
            "workload": "512 systems, N log-uniform [256, 16384], density U[0.2, 0.7], "
                        "kT U[0.5, 2], LJ or Yukawa, half with two-state reactions"}


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
    import numpy as np
    import torch
    from pyrdsim_gb300 import workloads
    from pyrdsim_gb300.engine import Engine
    torch.cuda.set_device(local)
    sd = workloads.active_wall_fluid(n=args.n, seed=2 + rank)
    eng = Engine([sd], device=local)
    N, seg = sd.n_particles, args.segment
    stream = torch.cuda.ExternalStream(eng.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    x0, t0 = eng.state()
    for _ in range(args.warmup):
        eng.step(seg)
    torch.cuda.synchronize()
    eng.profile()  # reset counters
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
    prof_counts = eng.profile()
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    ms_max = max_over_ranks(ms, ws)
    value = ws * N * seg * args.steps / (ms_max / 1e3)
    launches = sum(v["launches"] for k, v in prof_counts.items() if k != "hook")
    # roofline pass: per-kernel CUDA events on the engine stream
    eng.set_profiling(True)
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        eng.step(seg)
    torch.cuda.synchronize()
    prof = eng.profile()
    eng.set_profiling(False)
    f_ms = prof["force"]["ms"] / max(1, prof["force"]["timed"])
    r_ms = prof["react"]["ms"] / max(1, prof["react"]["timed"])
    peak, peak_kind = peaks()
    achieved = ALG_BYTES * N / (f_ms / 1e3) / 1e9
    traffic = traffic_per_launch(N)
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
                         "within a step", "parallelism": f"replicas x{ws}"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(N * 2 * 8 + N * 4),
                "d2h_bytes_per_step": int(N * 2 * 8 + N * 4),
                "path": "C ABI: rdsim_set_state (host) + rdsim_step + rdsim_get_state (host)"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "kernel": "k_force_l<2,2>",
                     "algorithmic_bytes_per_launch": ALG_BYTES * N,
                     "avg_launch_us": f_ms * 1e3, "peak_source": peak_kind,
                     "react_avg_launch_us": r_ms * 1e3},
        "kernel_ms": {k: v["ms"] for k, v in prof.items()},
        "kernel_launches": {k: v["launches"] for k, v in prof.items()},
        "clocks": clk,
        "engine": eng.info(),
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        try:
            out["cpu_baseline"] = cpu_baseline("active_wall_fluid")
        except Exception as exc:
            out["cpu_baseline"] = {"unavailable": str(exc)[:200]}
        try:
            out["force_err_vs_fp64"] = force_error(eng, sd, f"cuda:{local}")
        except Exception as exc:
            out["force_err_vs_fp64"] = {"unavailable": str(exc)[:200]}
    if rank == 0 and ws == 1 and not args.no_ensemble:
        eng.close()
        try:
            out["ensemble"] = ensemble_comparison(local)
        except Exception as exc:
            out["ensemble"] = {"unavailable": str(exc)[:200]}
    if rank == 0 and ws == 1 and not args.no_precision:
        try:
            out["precision_vs_fp64"] = precision_report(local)
        except Exception as exc:
            out["precision_vs_fp64"] = {"unavailable": str(exc)[:200]}
    if rank == 0 and ws == 1 and not args.no_adjoint:
        try:
            out["adjoint"] = adjoint_timing(local)
        except Exception as exc:
            out["adjoint"] = {"unavailable": str(exc)[:200]}
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
