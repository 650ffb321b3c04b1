#!/usr/bin/env python
"""Benchmark of the full-physics fire simulation step on GB300.

Workload: the 128x256x128 full-physics step (5 mm cells, 0.64 x 1.28 x 0.64 m, dt = 1/240 s, FP32) with
6 seeded pyrolysis spots of 1-4 g/s, vorticity confinement 0.3, curl-noise amplitude 0.2, soot forming
after a gas age of 20-60 ms, and the pressure solved each step to a 1e-5 relative residual (at most 8
V(2,2) cycles).  Synthetic: the state evolves from rest under the seeded emitter; no dataset is involved.

A step is one FireSim.step (src/sim.js:627-648): advection, forces, divergence, multigrid, projection.
  value      steps/s over the timed region (device time, CUDA events on the launching stream; inputs resident)
  e2e        steps/s through the C ABI with a host parameter update, the parameter-block upload and a
             device->host read of the step's diagnostics (S stats + heat release) every step (host clock;
             per-step diagnostics on, so the step graph forms them beside the pressure solve)
  roofline   the dominant stage's algorithmic bytes / its average duration, against measured HBM peak
  cpu_baseline  the CPU oracle (FP32, OpenMP on all host cores) on a bounded sample of the same workload

`--impl reference` times the CPU implementation of the step (the oracle port of the reference's WGSL; the
reference's own WebGPU step cannot run on this machine) on the same workload and prints the same line.
Multi-GPU (`torchrun --nproc-per-node N`): replicas only, one independent simulation per GPU; value is the
aggregate steps/s of all ranks over the max-over-ranks time.
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "procedural-fire_gb300"
for p in (PKG, ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

WORKLOAD = dict(
    name="fire-step-128x256x128-fp32", res=(128, 256, 128), size=(0.64, 1.28, 0.64), dt=1.0 / 240.0,
    spots=6, spot_seed=2, flux=(1.0, 4.0), sigma=0.02, radius=0.2, vortEps=0.3, turbAmp=0.2,
    soot_age=(0.02, 0.06), mg_tol=1e-5, mg_max_cycles=8, mg_omega=1.2, preroll=60,
)
METRIC = "steps/s, full-physics fire step at 128x256x128 (FP32)"

# Algorithmic bytes per cell of each stage: every array the stage must read once and write once (float4
# fields of 16 B, pressure/divergence of 4 B).  forces adds the 16 MiB curl table once per step.
B_ALG = {"adv1": 96.0, "adv2": 144.0, "forces": 112.0, "div": 20.0, "project": 40.0}
B_MG_CYCLE = 75.0      # V(2,2): level 0 (4 sweeps x 12 + restrict 9 + prolong 8.5) x 8/7 over the levels
FALLBACK_HBM_GBS = 6800.0


# ------------------------------------------------------------------------------------------ distributed
def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def dist_init(backend: str):
    import torch.distributed as dist
    rank, world, _ = dist_env()
    if world > 1 and not dist.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        os.environ.setdefault("MASTER_PORT", "29511")
        dist.init_process_group(backend, rank=rank, world_size=world)
    return rank, world


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def max_over_ranks(x: float, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------------------------------ clocks
class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        # raw samples (the JSON line carries their summary); FIRE_BENCH_CLOCKS_DIR keeps them where wanted
        out = os.environ.get("FIRE_BENCH_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = Path(out) / f"fire_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.path.parent.mkdir(parents=True, exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self, max_mhz_default=2070.0):
        rows = []
        try:
            for line in self.path.read_text().splitlines():
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                    rows.append(parts)
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": max_mhz_default, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows]
        mx = float(rows[0][2])
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        loaded = [s for s in sm if s > 0.5 * mx] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------------------------------------ helpers
def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(kernel_stage: str):
    """Per-launch DRAM bytes of a stage's kernel at the bench workload, from the committed ncu summary."""
    p = ROOT / "profiles" / "ncu_traffic.json"
    try:
        d = json.loads(p.read_text())
        v = d.get(WORKLOAD["name"], {}).get(kernel_stage)
        return None if v is None else float(v)
    except Exception:
        return None


def make_sim(F, device: int, mg_fixed: int = 0):
    """The workload's simulation.  mg_fixed > 0 replaces the residual-driven solve by that many fixed
    V-cycles (same kernels, no conditional graph node), which ncu needs to profile graph kernel nodes."""
    W = WORKLOAD
    sim = F.FireSim(res=W["res"], size=W["size"], logs=None, vcycles=mg_fixed or 4, device=device,
                    mg_max_cycles=0 if mg_fixed else W["mg_max_cycles"], mg_tol=W["mg_tol"])
    sim.set_params({"vortEps": W["vortEps"], "turbAmp": W["turbAmp"]})
    sim.set_soot_age(*W["soot_age"])
    sim.set_bed_gain(0.0)
    sim.set_spots(F.make_spots(W["spot_seed"], W["spots"], W["flux"][0], W["flux"][1], W["sigma"], W["radius"]))
    if not mg_fixed:
        sim.set_mg_omega(W["mg_omega"])   # over-relaxed fine-level smoothing: 3 cycles to 1e-5 instead of ~4.5
    return sim


def launches_per_step(sim, cycles_per_step: float) -> float:
    """Kernels launched per step by the captured graph: 5 stencil kernels (the divergence kernel also clears
    the solve's cycle count), and per V-cycle 10 per level above the shared-memory tail (2 + 2 red-black sweeps of 2 colour launches each,
    restriction, prolongation) less one per level below the finest (its first colour-0 sweep runs inside the
    restriction onto it), the tail kernel, the residual norm and the decision kernel.  The tail starts at the
    finest level that fits in 200 KB of shared memory (one CTA, or 8 CTAs with distributed levels) and has at
    most 8192 cells."""
    n = len(sim.levels)
    T = n
    for l in range(n - 1, -1, -1):
        nx, ny, nz = sim.levels[l]["dims"]
        cells = nx * ny * nz
        smem = 0
        for k in range(l, n):
            kx, ky, kz = sim.levels[k]["dims"]
            c = kx * ky * kz
            dist = k < n - 1 and kz % 16 == 0 and c >= 8 * 512
            smem += 8 * (c // 8 if dist else c)
        if cells <= 8192 and smem <= 200 * 1024:
            T = l
        else:
            break
    top = min(T, n - 1)
    per_cycle = 10 * top - max(top - 1, 0) + (1 if T < n else 0) + 2
    return 5 + per_cycle * cycles_per_step


def workload_config(preroll: int) -> dict:
    """The workload description both arms print (identical, so the two lines describe the same work)."""
    W = WORKLOAD
    return {"workload": W["name"], "grid": list(W["res"]), "cell_m": 0.005, "dt": W["dt"], "spots": W["spots"],
            "emitter": "6 seeded floor spots, flux U(1, 4) g/s, no logs, no coal bed",
            "mg": f"V(2,2), every sweep over-relaxed (omega {W['mg_omega']}), to {W['mg_tol']} rel. residual, "
                  f"max {W['mg_max_cycles']} cycles",
            "state": f"timed steps follow {preroll} preroll steps from rest",
            "l2": "inputs larger than L2 (fields ~740 MB vs 129 MB L2)"}


class OracleStepper:
    """The workload on the CPU oracle (FP32, OpenMP): the same seeded tables, spots, parameters, solver and
    per-step simulated time as the GPU arm.  Built from the oracle alone (no product library is loaded)."""

    def __init__(self, O, threads: int):
        W = WORKLOAD
        O.build()
        O.set_threads(threads)
        noise = O.noise_table(128, 1)
        self.O = O
        self.dx = np.float32(np.float64(np.float32(W["size"][0])) / W["res"][0])
        self.orc = O.OracleSim(W["res"], float(self.dx))
        self.orc.set_tables(noise, O.curl_table(noise))
        self.orc.set_logs(np.zeros(0, np.float32))
        self.orc.set_modes(omega=W["mg_omega"])
        self.blk = oracle_block(O)
        self.time, self.frame, self.geo = 0.0, 0, True
        self.cycles = []

    def step(self):
        W = WORKLOAD
        dt = np.float32(W["dt"])
        self.blk[5] = np.float32(self.time)      # time and frame as FireSim.uploadUniforms writes them (src/sim.js:620-624)
        self.blk[6] = np.float32(self.frame)
        self.orc.set_params(self.blk[:64])
        self.orc.set_ext(self.blk[64:])
        self.cycles.append(self.orc.step_raw(self.geo, -W["mg_max_cycles"], W["mg_tol"]))
        self.geo = False
        self.time += float(dt)
        self.frame += 1

    def load_state(self, sim):
        """Continues from a GPU simulation's state (fields, level-0 pressure, time and frame)."""
        for name in ("vel", "S", "S2", "geo"):
            self.orc.put(name, sim.download(name).astype(np.float32))
        self.orc.put_level(0, "p", sim.download("p").astype(np.float32).reshape(self.orc.levels[0][0][::-1]))
        info = sim.info()
        self.time, self.frame, self.geo = float(info.time), int(info.frame), False


def oracle_block(O):
    """The workload's 208-float block (SIM_FIELDS uniforms + extension) from the oracle's restatements of
    SIM_DEFAULTS and the seeded spots; the oracle recomputes the derived extension slots itself."""
    W = WORKLOAD
    names = ["nx", "ny", "nz", "dx", "dt", "time", "frame", "seed", "ox", "oy", "oz", "nLogs"]
    blk = np.zeros(208, np.float32)
    blk[:64] = O.sim_defaults()
    for i, v in enumerate(W["res"]):
        blk[i] = v
    size0 = np.float32(W["size"][0])
    blk[names.index("dx")] = np.float32(np.float64(size0) / W["res"][0])
    blk[names.index("dt")] = np.float32(W["dt"])
    blk[names.index("ox")] = np.float32(-size0 / np.float32(2))
    blk[names.index("oz")] = np.float32(-np.float32(W["size"][2]) / np.float32(2))
    blk[34] = W["vortEps"]     # SIM_FIELDS index of vortEps (src/sim.js:19)
    blk[35] = W["turbAmp"]     # turbAmp
    e = blk[64:]
    e[0], e[1], e[2], e[4] = W["soot_age"][0], W["soot_age"][1], 0.0, 4.0
    spots = O.make_spots(W["spot_seed"], W["spots"], W["flux"][0], W["flux"][1], W["sigma"], W["radius"])
    e[3] = len(spots)
    for i, sp in enumerate(spots):
        e[16 + 8 * i: 16 + 8 * i + 5] = sp
    return blk


def cpu_baseline(sim, steps: int = 2):
    """The oracle (FP32, OpenMP on all host threads) continuing the GPU simulation's developed state for
    `steps` steps of the same workload and solver."""
    import oracle as O
    threads = os.cpu_count() or 1
    ref = OracleStepper(O, threads)
    ref.load_state(sim)
    t0 = time.perf_counter()
    for _ in range(steps):
        ref.step()
    el = time.perf_counter() - t0
    return steps / el, threads, (f"{steps} steps of {WORKLOAD['res'][0]}x{WORKLOAD['res'][1]}x{WORKLOAD['res'][2]} continuing "
                                 f"the GPU run's developed state (after its timed steps), {np.mean(ref.cycles):.2f} V-cycles each")


# Standalone pressure solve: 256x512x256 cells at 5 mm, seeded zero-mean RHS of 32 Gaussian sources
# (sigma 1-4 cells, amplitude N(0,1)) plus 1e-3 white noise, solved from x = 0 to a 1e-6 relative residual.
POISSON = dict(name="poisson-256x512x256", res=(256, 512, 256), h=0.005, seed=3, sources=32, noise=1e-3, tol=1e-6)


def run_poisson(dev: int, reps: int = 3, fixed_iters: int = 0):
    """Times each form of the standalone solver on the POISSON workload (device time, CUDA events).  The
    FP32 form (the step's V-cycle on an FP32 x) cannot get below the FP32 representation floor of the
    solution (~2e-5 here); it is timed to 3e-5 and its floor reported.  fixed_iters > 0 (profiling aid)
    instead runs exactly that many iterations of each form once: the solve graph is then unrolled, with no
    conditional node, so every kernel can be profiled."""
    import torch
    import fire_sim as F
    P = POISSON
    if fixed_iters > 0:
        n = P["res"][0] * P["res"][1] * P["res"][2]
        b = torch.empty(n, dtype=torch.float32, device=f"cuda:{dev}")
        x, lo = torch.zeros_like(b), torch.zeros_like(b)
        out = {}
        for prec in ("fp32", "ir32", "fp16", "bf16"):
            ps = F.Poisson(P["res"], P["h"], prec, device=dev)
            ps.make_rhs(b, seed=P["seed"], n_sources=P["sources"], noise=P["noise"])
            x.zero_(); lo.zero_()
            ps.solve(b, x, tol=0.0, max_iters=fixed_iters, x_lo=lo)
            out[prec] = ps.result()
            ps.close()
        return {"workload": P["name"], "fixed_iterations": fixed_iters, "forms": out}
    n = P["res"][0] * P["res"][1] * P["res"][2]
    b = torch.empty(n, dtype=torch.float32, device=f"cuda:{dev}")
    x = torch.zeros_like(b)
    lo = torch.zeros_like(b)
    st = torch.cuda.current_stream(dev)
    forms = {}
    for prec in ("fp32", "ir32", "fp16", "bf16"):
        ps = F.Poisson(P["res"], P["h"], prec, device=dev)
        ps.make_rhs(b, seed=P["seed"], n_sources=P["sources"], noise=P["noise"])
        tol = 3e-5 if prec == "fp32" else P["tol"]
        times = []
        for r in range(reps + 1):
            x.zero_(); lo.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            ps.solve(b, x, tol=tol, max_iters=60, x_lo=lo, stream=st.cuda_stream)
            e1.record(st)
            res = ps.result()
            if r > 0:
                times.append(e0.elapsed_time(e1))
        forms[prec] = {"ms": statistics.median(times), "iterations": res["iterations"], "rel_residual": res["rel_residual"],
                       "tol": tol}
        if prec == "fp32":
            ps.solve(b, x, tol=0.0, max_iters=30, stream=st.cuda_stream)
            forms[prec]["floor_rel_residual"] = ps.result()["rel_residual"]
        ps.close()
    base = forms["ir32"]["ms"]
    return {"workload": P["name"], "grid": list(P["res"]), "tol": P["tol"], "rhs": "32 seeded Gaussian sources + 1e-3 noise, mean removed",
            "forms": forms, "speedup_vs_ir32": {k: base / forms[k]["ms"] for k in ("fp16", "bf16")},
            "note": "ir32/fp16/bf16: iterative refinement with FP32-pair x, level storage FP32/half/bfloat16, exact FP64 "
                    "coarsest solve; fp32: the step's V(2,2) cycle on an FP32 x (stalls at its representation floor)"}


# Ensemble: 64 independent fires, 16 each at 32x64x32, 48x96x48, 64x128x64 and 96x192x96 cells of 1.25 cm,
# each with its own seed and 2-8 spots of 1-4 g/s, 4 V(2,2) cycles per step, dt = 1/120 s.
ENSEMBLE = dict(name="ensemble-64-fires", grids=((32, 64, 32), (48, 96, 48), (64, 128, 64), (96, 192, 96)), per_grid=16,
                cell_m=0.0125, dt=1.0 / 120.0, vcycles=4, preroll=20)


def _ensemble_members():
    rng = np.random.default_rng(4)
    members = []
    for g in ENSEMBLE["grids"]:
        for k in range(ENSEMBLE["per_grid"]):
            size = tuple(ENSEMBLE["cell_m"] * v for v in g)
            members.append(dict(res=g, size=size, seed=1000 + len(members), spots=int(rng.integers(2, 9))))
    return members


def _ensemble_configure(sim, m, F):
    sim.set_spots(F.make_spots(m["seed"], m["spots"], 1.0, 4.0, 0.02, 0.3 * m["size"][0]))
    sim.set_params({"seed": float(m["seed"]), "vortEps": 0.3, "turbAmp": 0.2})
    sim.set_soot_age(0.02, 0.06)
    sim.set_bed_gain(0.0)


def run_ensemble(dev: int, steps: int = 20):
    """Aggregate cell updates/s of the 64-fire ensemble stepped by batched launches, against the same 64
    simulations stepped one after another (each its own per-step CUDA graph)."""
    import torch
    import fire_sim as F
    E = ENSEMBLE
    members = _ensemble_members()
    cells = sum(int(np.prod(m["res"])) for m in members)
    st = torch.cuda.current_stream(dev)
    ens = F.Ensemble(members, vcycles=E["vcycles"], device=dev)
    for s, m in zip(ens.members, members):
        _ensemble_configure(s, m, F)
    ens.step(E["dt"], E["preroll"], stream=st.cuda_stream)   # the autotuner runs on step 8 of these
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    ens.step(E["dt"], steps, stream=st.cuda_stream)
    e1.record(st)
    torch.cuda.synchronize(dev)
    ms_batched = e0.elapsed_time(e1) / steps
    tuned = ens.tiles()
    ens.set_tiles([0, 0, 0, 0, 0])   # the same ensemble with the untuned (per-simulation) tiles
    ens.step(E["dt"], 2, stream=st.cuda_stream)
    e0.record(st)
    ens.step(E["dt"], steps, stream=st.cuda_stream)
    e1.record(st)
    torch.cuda.synchronize(dev)
    ms_untuned = e0.elapsed_time(e1) / steps
    ens.close()
    sims = []
    for m in members:
        s = F.FireSim(res=m["res"], size=m["size"], vcycles=E["vcycles"], device=dev)
        _ensemble_configure(s, m, F)
        sims.append(s)
    for s in sims:
        s.step(E["dt"], E["preroll"], stream=st.cuda_stream)
    torch.cuda.synchronize(dev)
    e0.record(st)
    for _ in range(steps):
        for s in sims:
            s.step(E["dt"], 1, stream=st.cuda_stream)
    e1.record(st)
    torch.cuda.synchronize(dev)
    ms_single = e0.elapsed_time(e1) / steps
    for s in sims:
        s.close()
    return {"workload": E["name"], "members": len(members), "cells": cells, "steps": steps,
            "ms_per_step_batched": ms_batched, "ms_per_step_one_at_a_time": ms_single,
            "gcell_updates_per_s_batched": cells / (ms_batched * 1e-3) / 1e9,
            "gcell_updates_per_s_one_at_a_time": cells / (ms_single * 1e-3) / 1e9,
            "speedup": ms_single / ms_batched,
            "tiles": {"stages": ["adv1", "adv2", "forces", "div", "project"],
                      "chosen": tuned[0].tolist() if tuned else None,
                      "candidate_ms": tuned[1].round(5).tolist() if tuned else None,
                      "cell_tiles": ["32x4x2", "32x8x1", "32x2x4", "64x4x1"], "forces_depths": [16, 8, 32],
                      "ms_per_step_untuned_tiles": ms_untuned}}


# Inverse source fit through the discrete adjoint: 64x128x64 cells at 1 cm, dt = 1/120, 120 steps from rest,
# 8 floor spots.  The target is the final temperature and soot of a run with seed-A fluxes; the fit starts
# from seed-B fluxes at the same positions; checkpoints every 10 steps.
ADJOINT = dict(name="adjoint-fit-64x128x64", res=(64, 128, 64), size=(0.64, 1.28, 0.64), dt=1.0 / 120.0, steps=120,
               checkpoint=10, spots=8, seed_a=11, seed_b=12, sigma=0.02, radius=0.12, mg_tol=1e-5, mg_max_cycles=8,
               mg_omega=1.2, iterations=3)


def run_adjoint(dev: int, steps: int = 0, iterations: int = -1, mg_fixed: int = 0):
    """Adjoint cost per step on the source-fit workload (checkpoints every 10 steps, and with the whole
    rollout on the tape), then how far the gradient describes the loss: for rollouts of 10, 30 and 120 steps,
    the loss along -grad against the first-order prediction, and a fit of the fluxes on the horizon where the
    gradient is predictive (steps / iterations override the workload's for profiling runs)."""
    import torch
    import fire_sim as F
    A = dict(ADJOINT)
    if steps > 0:
        A["steps"] = steps
    if iterations >= 0:
        A["iterations"] = iterations
    st = torch.cuda.current_stream(dev)
    spots_a = F.make_spots(A["seed_a"], A["spots"], 1.0, 4.0, A["sigma"], A["radius"])
    spots_b = spots_a.copy()
    spots_b[:, 4] = F.make_spots(A["seed_b"], A["spots"], 1.0, 4.0, A["sigma"], A["radius"])[:, 4]

    def make(spots):
        s = F.FireSim(res=A["res"], size=A["size"], vcycles=mg_fixed or 4, device=dev,
                      mg_max_cycles=0 if mg_fixed else A["mg_max_cycles"], mg_tol=A["mg_tol"])
        s.set_params({"vortEps": 0.3, "turbAmp": 0.2})
        s.set_soot_age(0.02, 0.06)
        s.set_bed_gain(0.0)
        s.set_spots(spots)
        if not mg_fixed:
            s.set_mg_omega(A["mg_omega"])
        return s

    def target_at(n):
        s = make(spots_a)
        s.step(A["dt"], n, stream=st.cuda_stream)
        out = s.download("S").astype(np.float32)
        s.close()
        return out

    def run(adj, sim, flux, target):
        sim.reset()
        sp = spots_b.copy()
        sp[:, 4] = flux
        sim.set_spots(sp)
        adj.forward(A["dt"], stream=st.cuda_stream)
        return adj.loss(target)

    # cost: the plain forward (the step graph, same solve), the taped forward and the backward.  One step
    # first builds the simulation's graph (its capture and instantiation stay out of the timing), then the
    # timed rollout starts from rest.
    sim = make(spots_a)
    sim.step(A["dt"], 1, stream=st.cuda_stream)
    torch.cuda.synchronize(dev)
    sim.reset()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    sim.step(A["dt"], A["steps"], stream=st.cuda_stream)
    e1.record(st)
    torch.cuda.synchronize(dev)
    ms_plain = e0.elapsed_time(e1) / A["steps"]
    target = sim.download("S").astype(np.float32)
    sim.close()
    sim = make(spots_b)
    fwd, bwd = [], []
    for ck in (A["checkpoint"], A["steps"]):
        adj = F.Adjoint(sim, A["steps"], ck)
        for _ in range(2):
            run(adj, sim, spots_b[:, 4], target)
            adj.backward(stream=st.cuda_stream)
            f_ms, b_ms = adj.timing()
        fwd.append(f_ms / A["steps"])
        bwd.append(b_ms / A["steps"])
        adj.close()
    # how far the gradient describes the loss, per rollout length
    horizons = []
    fit = []
    for n in sorted({10, 30, A["steps"]}):
        tgt = target_at(n)
        adj = F.Adjoint(sim, n, min(A["checkpoint"], n))
        flux0 = spots_b[:, 4].astype(np.float64)
        L0 = run(adj, sim, flux0, tgt)
        adj.backward(stream=st.cuda_stream)
        g = adj.grad_spots(A["spots"])
        d = -g / max(np.linalg.norm(g), 1e-30)
        probe = []
        for s in (1e-4, 1e-3, 1e-2, 1e-1):
            L = run(adj, sim, np.clip(flux0 + s * d, 0.0, 8.0), tgt)
            probe.append({"step_gps": s, "loss_change": L - L0, "predicted_change": s * float(g @ d)})
        horizons.append({"steps": n, "loss": L0, "grad_norm": float(np.linalg.norm(g)), "along_minus_grad": probe})
        if n == 10 and A["iterations"] > 0:
            # projected gradient descent on the fluxes with backtracking, on this horizon
            flux, L = flux0.copy(), L0
            fit.append({"loss": L, "flux_err_gps": float(np.abs(flux - spots_a[:, 4]).max())})
            for _ in range(A["iterations"]):
                run(adj, sim, flux, tgt)
                adj.backward(stream=st.cuda_stream)
                g = adj.grad_spots(A["spots"])
                step = 0.5
                for _ in range(6):
                    trial = np.clip(flux - step * g / max(np.linalg.norm(g), 1e-30), 0.0, 8.0)
                    Lt = run(adj, sim, trial, tgt)
                    if Lt < L:
                        flux, L = trial, Lt
                        break
                    step *= 0.25
                fit.append({"loss": L, "flux_err_gps": float(np.abs(flux - spots_a[:, 4]).max())})
        adj.close()
    sim.close()
    return {"workload": A["name"], "steps": A["steps"], "checkpoint_every": A["checkpoint"],
            "mg": f"{mg_fixed} fixed V(2,2) cycles" if mg_fixed else
                  f"V(2,2), omega {A['mg_omega']}, to {A['mg_tol']} rel. residual, max {A['mg_max_cycles']}",
            "ms_per_step_forward_plain": ms_plain, "ms_per_step_forward_taped": fwd[0],
            "ms_per_step_backward": bwd[0], "adjoint_over_forward": bwd[0] / ms_plain,
            "ms_per_step_backward_whole_tape": bwd[1], "adjoint_over_forward_whole_tape": bwd[1] / ms_plain,
            "backward_includes": "recompute of every segment but the last from its checkpoint, then the reverse steps",
            "gradient_vs_horizon": horizons, "fit_10_steps": fit}


# Consumers of the step on the throughput workload's state: the sparks update (8192 sparks, the page's count,
# src/main.js:42), the renderer's fire passes into a headless image at the page's 960x1080 view and the
# 1080x1920 capture size (src/main.js:53-54, 161) with volume scale 1, and the cinematic's capture-mode driver.
CONSUMERS = dict(name="consumers-128x256x128", sparks=8192, views=((960, 1080), (1080, 1920)), vol_scale=1.0, reps=20)


def run_consumers(dev: int):
    """Device time per call of the sparks step and the volume render, and capture-mode steps/s."""
    import torch
    import fire_sim as F
    C, W = CONSUMERS, WORKLOAD
    st = torch.cuda.current_stream(dev)
    sh = st.cuda_stream
    sim = make_sim(F, dev)
    sim.step(W["dt"], W["preroll"], stream=sh)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize(dev)
        e0.record(st)
        for _ in range(reps):
            fn()
        e1.record(st)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / reps

    out = {"workload": C["name"]}
    sp = F.Sparks(sim, C["sparks"])
    sp.set(rate=60.0)
    for _ in range(30):
        sp.burst(n=120, pos=(0.0, 0.1, 0.0))
        sp.step(W["dt"], stream=sh)
    alive = int((sp.download()[:, 14] > 0.5).sum())
    out["sparks"] = {"count": C["sparks"], "alive": alive, "ms_per_step": timed(lambda: sp.step(W["dt"], stream=sh), 200)}
    sp.close()
    views = []
    for w, h in C["views"]:
        vol = F.Volume(sim, width=w, height=h, vol_scale=C["vol_scale"])
        vol.set_camera((0.45, 0.45, 1.1), (0.0, 0.35, 0.0), 40.0)
        frame = [0]

        def render():
            frame[0] += 1
            vol.render(1.0 + frame[0] / 30.0, frame[0], stream=sh)

        ms = timed(render, C["reps"])
        views.append({"image": [vol.vw, vol.vh], "ms_per_frame": ms, "mrays_per_s": vol.vw * vol.vh / (ms * 1e-3) / 1e6})
        vol.close()
    out["volume"] = views
    sim.close()
    # capture mode: timeline.capStep (parameters, log offsets, bursts) + the simulation and spark steps
    sim = make_sim(F, dev)
    sp = F.Sparks(sim, C["sparks"])
    tl = F.Timeline(F.build_campfire(7), 8)
    for j in range(24):
        tl.step(sim, j, sp, stream=sh)
    torch.cuda.synchronize(dev)
    n = 120
    t0 = time.perf_counter()
    for j in range(24, 24 + n):
        tl.step(sim, j, sp, stream=sh)
    torch.cuda.synchronize(dev)
    out["timeline_capture"] = {"steps_per_frame": 8, "capture_steps_per_s": n / (time.perf_counter() - t0),
                               "note": "host clock, timeline cues + simulation + sparks per step"}
    tl.close()
    sp.close()
    sim.close()
    return out


# ------------------------------------------------------------------------------------------ arms
def run_ours(args):
    import torch
    import fire_sim as F
    rank, world, local = dist_env()
    if world > 1:
        torch.cuda.set_device(local)
        dist_init("nccl")
    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    W = WORKLOAD
    cells = W["res"][0] * W["res"][1] * W["res"][2]
    sim = make_sim(F, dev, args.mg_fixed)
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    dt = W["dt"]

    sim.step(dt, args.preroll + args.warmup, stream=sh)
    torch.cuda.synchronize(dev)
    info0 = sim.info()
    # the state the timed steps start from: the per-stage profile and the end-to-end loop below replay the
    # same steps from it, so all three numbers describe the same stretch of the fire's development
    start = sim.save()

    # ---- timed region: K steps, inputs resident in HBM (the fields exceed L2 several times over)
    sampler = ClockSampler(dev) if rank == 0 else None
    if sampler:
        sampler.__enter__()
    barrier()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sim.step(dt, args.steps, stream=sh)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    if sampler:
        sampler.__exit__()
    ms = e0.elapsed_time(e1)
    ms_max = max_over_ranks(ms, device=torch.device("cuda", dev))
    info1 = sim.info()
    cycles = (info1.total_cycles - info0.total_cycles) / max(args.steps, 1)
    value = world * args.steps / (ms_max / 1e3)

    # ---- per-stage profile (graph with event nodes between stages), averaged over the timed steps
    nprof = max(3, args.steps)
    sim.load(start)
    sim.profile(True)
    acc = {}
    for _ in range(nprof):
        sim.step(dt, 1, stream=sh)
        for k, v in sim.stage_times().items():
            acc[k] = acc.get(k, 0.0) + v / nprof
    sim.profile(False)

    # ---- end to end through the C ABI: host param update + block upload + stats readback per step
    pinned = torch.empty(17, dtype=torch.float64, pin_memory=True)
    sim.set_step_stats(True)      # each step's graph forms the diagnostics beside the pressure solve
    sim.step(dt, 1, stream=sh)    # builds that graph outside the timing
    sim.load(start)
    torch.cuda.synchronize(dev)
    barrier()
    t0 = time.perf_counter()
    for s in range(args.steps):
        sim.set_params({"windX": 0.05 * np.sin(0.01 * s)})
        sim.step(dt, 1, stream=sh)
        sim.stats_async(pinned.data_ptr(), stream=sh)
    torch.cuda.synchronize(dev)
    e2e_s = max_over_ranks(time.perf_counter() - t0, device=torch.device("cuda", dev))
    barrier()
    e2e = world * args.steps / e2e_s
    diag = pinned.numpy().copy()

    if rank != 0:
        return None

    # ---- roofline of the dominant single-kernel stage
    peak, peak_kind = measured_peak()
    stage_bytes = {k: B_ALG[k] * cells for k in B_ALG}
    stage_bytes["forces"] += 128 ** 3 * 8
    single = {k: acc[k] for k in B_ALG}
    dom = max(single, key=single.get)
    achieved = stage_bytes[dom] / (single[dom] * 1e-3) / 1e9
    mg_ms = acc["vcycle"]
    mg_gbs = B_MG_CYCLE * cycles * cells / (mg_ms * 1e-3) / 1e9 if mg_ms > 0 else None
    step_bytes = sum(stage_bytes.values()) + B_MG_CYCLE * cycles * cells
    traffic = ncu_traffic(dom)

    # ---- CPU baseline: oracle on a bounded sample
    cpu = None
    if world == 1 and not args.no_cpu:
        v, cores, sample = cpu_baseline(sim, steps=2)
        cpu = {"value": v, "unit": "steps/s", "cores": cores, "kind": "port", "sample": sample}

    clocks = sampler.summary() if sampler else None
    out = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args.preroll),
        "parallelism": f"replicas x{world}", "mean_vcycles_per_step": cycles,
        "gcell_updates_per_s": value * cells / 1e9,
        "e2e": {"value": e2e, "unit": "steps/s", "h2d_bytes_per_step": 208 * 4, "d2h_bytes_per_step": 17 * 8},
        "gpu_launches": int(round(args.steps * launches_per_step(sim, cycles))),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "bytes_per_cell": B_ALG[dom] + (128 ** 3 * 8 / cells if dom == "forces" else 0.0)},
        "stage_ms": {k: round(v, 5) for k, v in acc.items()},
        "step_roofline": {"alg_bytes_per_step": step_bytes, "achieved_gbs": step_bytes / (ms_max / args.steps * 1e-3) / 1e9,
                          "frac": step_bytes / (ms_max / args.steps * 1e-3) / 1e9 / peak, "mg_gbs": mg_gbs},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "diag_last_step": {"hrr_kw": float(diag[16]), "T_max": 293.0 + 1000.0 * float(diag[1])},
        "poisson": None,
    }
    out["ensemble"] = None
    out["adjoint"] = None
    out["consumers"] = None
    if world == 1 and not (args.no_poisson and args.no_ensemble and args.no_adjoint and args.no_consumers):
        sim.close()   # frees the step's arena before the standalone workloads
        if not args.no_poisson:
            out["poisson"] = run_poisson(dev)
        if not args.no_ensemble:
            out["ensemble"] = run_ensemble(dev)
        if not args.no_adjoint:
            out["adjoint"] = run_adjoint(dev)
        if not args.no_consumers:
            out["consumers"] = run_consumers(dev)
    return out


def run_reference(args):
    """The CPU implementation of the step (the oracle port of the reference's WGSL, FP32, all host threads) on
    the same workload: the same preroll from rest, solver and per-step time; then `steps` timed steps (fewer
    if a step is slow, within a fixed budget).  Loads no product library."""
    rank, world, _ = dist_env()
    if rank != 0:
        return None
    import oracle as O
    threads = os.cpu_count() or 1
    ref = OracleStepper(O, threads)
    for _ in range(args.preroll + args.warmup):
        ref.step()
    t_step = None
    t0 = time.perf_counter()
    ref.step()
    t_step = time.perf_counter() - t0
    budget = 120.0
    k = max(2, min(args.steps, int(budget / max(t_step, 1e-3))))
    n0 = len(ref.cycles)
    t0 = time.perf_counter()
    for _ in range(k):
        ref.step()
    el = time.perf_counter() - t0
    v = k / el
    cycles = float(np.mean(ref.cycles[n0:]))
    return {
        "metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": world, "steps": k, "warmup": args.warmup,
        "ms_per_step": 1e3 * el / k, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic", "impl": "reference", "config": workload_config(args.preroll),
        "parallelism": "CPU, one process", "mean_vcycles_per_step": cycles,
        "gcell_updates_per_s": v * np.prod(WORKLOAD["res"]) / 1e9,
        "cpu_baseline": {"value": v, "unit": "steps/s", "cores": threads, "kind": "port",
                         "sample": f"{k} timed steps after {args.preroll} preroll + {args.warmup + 1} warm-up steps from rest, "
                                   f"{cycles:.2f} V-cycles each (the reference's WebGPU step needs a browser GPU stack, "
                                   f"unavailable on this box; this is the oracle's C++ restatement of its WGSL)"},
        "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline sample")
    ap.add_argument("--preroll", type=int, default=WORKLOAD["preroll"], help="untimed steps that develop the fire")
    ap.add_argument("--no-poisson", action="store_true", help="skip the standalone 256x512x256 pressure-solve timings")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the 64-fire ensemble timings")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint source-fit timings")
    ap.add_argument("--no-consumers", action="store_true", help="skip the sparks / volume / capture-mode timings")
    ap.add_argument("--only", choices=["poisson", "ensemble", "adjoint", "consumers"],
                    help="run just one of the side workloads and print its block (profiling aid)")
    ap.add_argument("--adjoint-steps", type=int, default=0, help="override the adjoint rollout length")
    ap.add_argument("--adjoint-iters", type=int, default=-1, help="override the number of fit iterations")
    ap.add_argument("--poisson-iters", type=int, default=0,
                    help="profiling aid for --only poisson: exactly N iterations per form, unrolled graphs")
    ap.add_argument("--mg-fixed", type=int, default=0,
                    help="profiling aid: N fixed V-cycles per step instead of the residual-driven solve")
    args = ap.parse_args(argv)
    args.warmup = max(args.warmup, 3)
    if args.only:
        import torch
        torch.cuda.init()
        fn = {"poisson": lambda: run_poisson(0, fixed_iters=args.poisson_iters), "ensemble": lambda: run_ensemble(0),
              "adjoint": lambda: run_adjoint(0, args.adjoint_steps, args.adjoint_iters, args.mg_fixed),
              "consumers": lambda: run_consumers(0)}[args.only]
        print(json.dumps({args.only: fn()}), flush=True)
        return
    out = run_reference(args) if args.impl == "reference" else run_ours(args)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
