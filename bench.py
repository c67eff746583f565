#!/usr/bin/env python3
"""Throughput of the GB300 Brownian-dynamics step, one JSON line on stdout.

Metric: particle-steps/s (live particles advanced per second, summed over
steps), the reference's benchmark quantity (particles.cpp:213-226 times
update() over N particles and I iterations).

Headline workload ("c3"): the plain 16M-particle, 8-species network in a
200 um reflecting cube with 12 reactions (dt 1 ms), seeded synthetic
positions.  The state (16M x 16 B = 256 MB) is larger than the 129 MB L2,
so no flush is needed between timed steps.  `value` is timed on the device
with CUDA events on the library's own stream over exactly --steps graph
launches after --warmup untimed ones; `e2e` runs the same workload through
the public C ABI with host buffers (upload, one step + a live-count readback
per step, download); `batched` times the 256-instance ensemble (c4) as one
pipeline per step and the same instances stepped one by one as plain systems.

--impl reference times the CPU restatement of the reference's step (the
reference has no CPU step of its own and its CUDA 2.x code does not build
with CUDA 13) on all host cores, on the headline workload itself; its
inputs are derived by oracle.params, so that arm never loads the GPU
library.

Multi-GPU (--gpus N under torchrun): instances are independent, so each
rank advances its own replica of the workload on its own GPU; the ranks only
meet at the barriers around the timed region (no data-path collective).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s plain vs batched ensemble on 1 GB300 at <1% rate/MSD error; p99"
T_START = time.perf_counter()


def progress(what):
    """One line on stderr per bench section (stdout carries only the JSON)."""
    print(f"[bench {time.perf_counter() - T_START:7.1f} s] {what}", file=sys.stderr, flush=True)
UNIT = "particle-steps/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1000)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="c3", choices=["c3", "c2"])
    p.add_argument("--n", type=int, default=0, help="override the particle count (debug)")
    p.add_argument("--no-batched", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-serving", action="store_true")
    p.add_argument("--no-surfaces", action="store_true")
    p.add_argument("--serve-jobs", type=int, default=200)
    p.add_argument("--profile-only", action="store_true", help="build + a few steps (for ncu)")
    p.add_argument("--profile-surfaces", action="store_true",
                   help="with --profile-only: the c3 step inside the cell (k_bin_surface)")
    return p.parse_args()


# ------------------------------------------------------------- distribution
class Dist:
    def __init__(self, want):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v):
        if not self.pg:
            return v
        import torch

        t = torch.tensor([float(v)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v):
        if not self.pg:
            return v
        import torch

        t = torch.tensor([float(v)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.proc:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


# ---------------------------------------------------------------- roofline
def measured_peak():
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_from_profiles(kernel, workload):
    """DRAM bytes per launch of `kernel` and where the figure comes from, read
    from the data file beside the committed ncu summaries (None when the
    kernel was not captured)."""
    try:
        d = json.load(open(os.path.join(ROOT, "profiles", "dram_traffic.json")))
        e = d[workload][kernel]
    except (OSError, KeyError, ValueError):
        return None, None
    src = (f"ncu capture at {e['capture_particles']} particles scaled x{e['scale']} to the workload "
           f"(profiles/{e['summary']})")
    return float(e["bytes_per_launch"]), src


def algorithmic_bytes(kernel, n_in, n_out, n_cells, binned=True):
    """Bytes a kernel must move at minimum (16-byte records, 4-byte cell words)."""
    table = {
        "k_bin": 16 * n_in + 16 * n_out + 4 * n_cells,      # read records, write bins, histogram
        "k_count": 16 * n_in + 4 * n_cells,                 # read records, write histogram
        "k_scan": 8 * n_cells,                               # read counts, write starts
        "k_scatter": 16 * n_in + 16 * n_out + 8 * n_cells,   # read + write records, starts + counts
        # read + write records, starts (+ clear the bin counts)
        "k_pairs_cells": 32 * n_out + (8 if binned else 4) * n_cells,
        "k_diffuse": 32 * n_in,
    }
    return table.get(kernel)


# -------------------------------------------------------------- workloads
def workload_desc(name, n_override=0):
    if name == "c3":
        n = n_override or 16_000_000
        side = 200.0 * (n / 16_000_000) ** (1 / 3)
        return f"c3: {n} particles, 8 species, 12 reactions, {side:.1f} um reflecting cube, dt 1 ms"
    n = n_override or 1_000_000
    side = 60.0 * (n / 1_000_000) ** (1 / 3)
    return f"c2: {n} particles, A+B<->C, {side:.1f} um cube, dt 0.5 ms"


def build_workload(name, n_override=0, normals="boxmuller", device=0, host_only=False):
    from gpusmoldyn_gb300 import configs

    dev = -1 if host_only else device
    if name == "c3":
        n = n_override or 16_000_000
        side = 200.0 * (n / 16_000_000) ** (1 / 3)
        return configs.build_c3(n=n, side=side, normals=normals, device=dev), workload_desc(name, n)
    n = n_override or 1_000_000
    side = 60.0 * (n / 1_000_000) ** (1 / 3)
    return configs.build_c2(n_a=n // 2, n_b=n - n // 2, side=side, normals=normals, device=dev), \
        workload_desc(name, n)


def network_and_particles(name, n_override, device):
    """A finalized handle without particles, and the initial state as host arrays."""
    from gpusmoldyn_gb300 import configs

    if name == "c3":
        n = n_override or 16_000_000
        side = 200.0 * (n / 16_000_000) ** (1 / 3)
        s = configs.c3_system(n=n, side=side, device=device)
        pos, sp = configs.c3_particles(n, side)
    else:
        n = n_override or 1_000_000
        side = 60.0 * (n / 1_000_000) ** (1 / 3)
        s = configs.c2_system(side=side, device=device)
        pos, sp = configs.c2_particles(n // 2, n - n // 2, side)
    return s, pos, sp


def oracle_c3(n, threads, seed=3):
    """The c3 workload at n particles (c3 density) for the CPU oracle: its
    inputs (grid, probabilities, radii, Poisson CDFs) are derived by
    oracle.params from the network description, so libgpusmoldyn.so is never
    loaded.  Returns the oracle, the initial records and the cube side."""
    from gpusmoldyn_gb300 import configs
    from oracle import params as oparams
    from oracle import py as orc

    side = 200.0 * (n / 16_000_000) ** (1 / 3)
    D, rx, _ = configs.c3_reactions(n / side ** 3)
    reactions = [oparams.Reaction(order, rc, pr, k) for order, rc, pr, k in rx]
    o = orc.OracleSystem.from_network(D, reactions, (0.0, 0.0, 0.0), (side, side, side), 1e-3, seed, n,
                                      normal_mode=0, threads=threads)
    pos, sp = configs.c3_particles(n, side, seed)
    return o, orc.records(pos, sp), side


def cpu_oracle_rate(n, steps, threads, budget_s=None, warmup=1):
    """Particle-steps/s of the CPU restatement on the c3 workload at n
    particles: `warmup` untimed steps, then up to `steps` timed ones (fewer
    when `budget_s` runs out)."""
    import numpy as np

    o, recs, side = oracle_c3(n, threads)
    cap = n + n // 8 + 65536
    for t in range(warmup):
        recs = o.step(t, recs, cap=cap)["recs"]
    done = 0
    psteps = 0
    t0 = time.perf_counter()
    for t in range(warmup, warmup + steps):
        live = int(np.sum(recs[:, 3] != 0xFFFFFFFF))
        recs = o.step(t, recs, cap=cap)["recs"]
        psteps += live
        done += 1
        if budget_s and time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    return psteps / el, done, el, side


def run_reference(args, dist):
    """The reference's step on the host cores: the oracle (the reference has
    no CPU step and its CUDA 2.x code does not build), all host threads, on
    the headline workload itself -- every step is a full step of the c3
    configuration."""
    if dist.rank != 0:
        return None
    threads = os.cpu_count() or 1
    n = args.n or 16_000_000
    warmup = max(args.warmup, 1)
    rate, done, el, side = cpu_oracle_rate(n, args.steps, threads, warmup=warmup)
    sample = (f"the full workload: c3, {n} particles in a {side:.1f} um cube, {done} steps ({el:.1f} s) after "
              f"{warmup} warm-up, OpenMP {threads} threads; inputs derived by oracle.params (no GPU library)")
    return {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus,
        "steps": done, "warmup": warmup, "ms_per_step": el / max(done, 1) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Philox uniform positions)",
        "config": {"workload": workload_desc("c3", args.n), "parallelism": f"cpu, {threads} threads",
                   "particles": n},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_gb300(args, dist):
    import numpy as np

    import gpusmoldyn_gb300
    from gpusmoldyn_gb300 import build as libbuild
    from gpusmoldyn_gb300 import configs

    libbuild.build()
    gpusmoldyn_gb300.load()
    device = dist.local
    if args.profile_only and args.profile_surfaces:
        n = args.n or 16_000_000
        s = configs.build_c3(n=n, side=200.0 * (n / 16_000_000) ** (1 / 3), surfaces=True, device=device)
        s.step(args.warmup + 3)
        s.synchronize()
        print(json.dumps({"profile_only": True, "surfaces": True, "n": s.count()}))
        s.close()
        return None
    # ---------------- headline: device-timed plain step
    progress("headline step")
    s, desc = build_workload(args.workload, args.n, device=device)
    s.step(args.warmup)
    s.synchronize()
    n0 = s.count()
    dims, cell, inv = s.grid()
    n_cells = int(np.prod(dims.astype(np.int64)))
    if args.profile_only:
        s.step(3)
        s.synchronize()
        print(json.dumps({"profile_only": True, "n": n0}))
        return None
    clocks = ClockSampler(device)
    dist.barrier()
    clocks.start()
    time.sleep(0.3)
    ms = s.time_steps(args.steps)
    clk = clocks.stop()
    dist.barrier()
    n1 = s.count()
    ms_max = dist.max(ms)
    local_ps = args.steps * 0.5 * (n0 + n1)
    total_ps = dist.sum(local_ps)
    value = total_ps / (ms_max / 1e3)
    kps = s.kernels_per_step()
    # per-kernel device times (events between kernels, outside the timed region)
    prof_steps = 20
    prof = s.profile_steps(prof_steps)
    dom = max(prof, key=prof.get)
    n_now = s.count()
    binned = "k_bin" in prof
    alg = algorithmic_bytes(dom, n_now, n_now, n_cells, binned)
    peak, peak_kind = measured_peak()
    roof = None
    if alg:
        achieved = alg / (prof[dom] / prof_steps / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind,
                "algorithmic_bytes_per_launch": alg}
        roof["traffic"], roof["traffic_source"] = traffic_from_profiles(dom, args.workload)
    step_alg = sum(v for v in (algorithmic_bytes(k, n_now, n_now, n_cells, binned) for k in prof) if v)
    step_roof = {"bytes_per_step": step_alg, "achieved_gbs": step_alg / (ms / args.steps / 1e3) / 1e9,
                 "frac": step_alg / (ms / args.steps / 1e3) / 1e9 / peak}
    s.close()

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Philox uniform positions)",
        "config": {"workload": desc, "particles": int(n0) * dist.world,
                   "parallelism": f"replicas x{dist.world}" if dist.world > 1 else "single GPU",
                   "particles_end": int(n1) * dist.world, "sort": "binned" if binned else "compact",
                   "normals": "box-muller (Philox)", "cells": n_cells, "l2": "state 256 MB > 129 MB L2, no flush"},
        "clocks": clk, "gpu_launches": kps * args.steps,
        "kernel_ms_per_step": {k: v / prof_steps for k, v in prof.items()},
        "roofline": roof, "step_roofline": step_roof,
    }

    # ---------------- end to end through the C ABI with host buffers
    progress('end to end through the C ABI with host buffers')
    if not args.no_e2e:
        s3, pos, sp = network_and_particles(args.workload, args.n, device)
        # the caller's arrays in the reference's layout (float4 positions, int
        # species) in pinned host memory, and the arrays it reads the result
        # into, kept across calls (as the reference's m_hPos / m_hTypes)
        pos4 = pinned((len(sp), 4), np.float32)
        pos4[:, :3] = pos
        pos4[:, 3] = 0.0
        sp4 = pinned((len(sp),), np.int32)
        sp4[:] = sp
        sp = sp4
        out4 = (pinned((2 * len(sp), 4), np.float32), pinned((2 * len(sp),), np.int32))
        # a first upload and readback, untimed, allocate the handle's buffers
        # (state, bins, pairs, transfer scratch), as a caller does once per
        # handle; the timed run then uploads its inputs into them
        tc = time.perf_counter()
        s3.set_particles(pos4, sp)
        cold_upload = time.perf_counter() - tc
        s3.particles4(out=out4)
        dist.barrier()
        t0 = time.perf_counter()
        s3.set_particles(pos4, sp)
        ta = time.perf_counter()
        psteps = 0
        live = len(sp)
        for _ in range(args.steps):
            s3.step(1)
            live = s3.count()
            psteps += live
        tb = time.perf_counter()
        pos_out, sp_out = s3.particles4(out=out4)
        t1 = time.perf_counter()
        dist.barrier()
        e2e_s = dist.max(t1 - t0)
        out["e2e"] = {"value": dist.sum(psteps) / e2e_s, "unit": UNIT,
                      "h2d_bytes_per_step": 20 * len(sp) / args.steps,
                      "d2h_bytes_per_step": 8 + 20 * len(sp_out) / args.steps,
                      "path": "bd_set_particles + steps x (bd_step(1) + bd_get_count) + bd_get_particles, pinned host "
                              "arrays, on a handle whose buffers an untimed first upload allocated",
                      "seconds": {"set_particles": ta - t0, "steps": tb - ta, "get_particles": t1 - tb,
                                  "first_upload_untimed": cold_upload}}
        s3.close()

    # ---------------- the same step with surfaces (c3 inside a cell)
    progress('the same step with surfaces')
    if not args.no_surfaces and args.workload == "c3":
        out["surfaces"] = run_surfaces(args, dist, device, out["value"])

    # ---------------- batched ensemble vs the plain per-instance loop
    progress('batched ensemble vs the plain per-instance loop')
    if not args.no_batched:
        out["batched"] = run_batched(args, dist, device)

    # ---------------- serving: continuous batching of c5-style requests
    progress('serving: continuous batching of c5-style requests')
    if not args.no_serving and dist.rank == 0:
        out["serving"] = run_serving(args, device)

    # ---------------- CPU baseline (rank 0, N = 1 only)
    progress('CPU baseline')
    if not args.no_cpu and dist.rank == 0 and dist.world == 1:
        threads = os.cpu_count() or 1
        n = args.n or 16_000_000
        rate, done, el, side = cpu_oracle_rate(n, 30, threads, budget_s=12.0)
        out["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": f"the c3 workload itself ({n} particles in a {side:.1f} um cube), {done} "
                                         f"steps ({el:.1f} s) after 1 warm-up, OpenMP {threads} threads"}
        # one step of the same workload on one core
        rate1, done1, el1, _ = cpu_oracle_rate(n, 1, 1, warmup=0)
        out["cpu_baseline"]["single_core"] = {"value": rate1, "unit": UNIT, "cores": 1,
                                              "sample": f"the same workload, {done1} step ({el1:.1f} s), 1 thread"}
    return out


def pinned(shape, dtype):
    """A numpy array over page-locked host memory (host<->device copies from
    and into it run at the link's DMA rate instead of being staged)."""
    import numpy as np
    import torch

    tdt = {np.float32: torch.float32, np.int32: torch.int32}[dtype]
    return torch.empty(shape, dtype=tdt, pin_memory=True).numpy()


def run_surfaces(args, dist, device, plain_value):
    """The c3 step inside a cell: a spherical membrane (one sphere panel) and
    a nucleus of 1280 triangles, walked by every diffusion step."""
    from gpusmoldyn_gb300 import configs

    n = args.n or 16_000_000
    side = 200.0 * (n / 16_000_000) ** (1 / 3)
    s = configs.build_c3(n=n, side=side, surfaces=True, device=device)
    s.step(args.warmup)
    s.synchronize()
    steps = max(args.steps // 4, 20)
    n0 = s.count()
    ms = s.time_steps(steps)
    n1 = s.count()
    value = dist.sum(steps * 0.5 * (n0 + n1)) / (dist.max(ms) / 1e3)
    prof = s.profile_steps(10)
    n_surf, n_panels = s.surface_counts()
    s.close()
    return {"workload": f"c3 inside a cell: {n} particles, {n_panels} panels in {n_surf} surfaces "
                        "(reflecting membrane crossed by S0 and S1, nucleus of 1280 triangles)",
            "value": value, "unit": UNIT, "steps": steps, "ms_per_step": ms / steps,
            "vs_plain_step": value / plain_value, "kernel_ms_per_step": {k: v / 10 for k, v in prof.items()}}


def run_batched(args, dist, device):
    """c4: 256 instances of the c2 network as one pipeline per step.  Under
    torchrun the instances are split across ranks by particle count
    (sharding.my_instances, no communication); each rank tunes the cell
    occupancy and launch shape on a scaled copy of its share (every 8th
    instance), then runs the c4-specified 2,000 steps.  The same instances
    are also stepped one after another as plain systems."""
    import numpy as np

    from gpusmoldyn_gb300 import configs, sharding, tune
    from gpusmoldyn_gb300.system import System

    inst_all, counts_all = configs.c4_instances()
    pos_all, sp_all = configs.c4_positions(inst_all, counts_all)
    offs = np.concatenate([[0], np.cumsum(counts_all)])
    mine = sharding.my_instances(counts_all, dist.world, dist.rank)

    def share(ids):
        inst = [inst_all[k] for k in ids]
        counts = np.array([counts_all[k] for k in ids], np.int64)
        pos = np.concatenate([pos_all[offs[k]:offs[k + 1]] for k in ids])
        sp = np.concatenate([sp_all[offs[k]:offs[k + 1]] for k in ids])
        return inst, counts, pos, sp

    def build(ids, occupancy=0.0):
        inst, counts, pos, sp = share(ids)
        s = System(dt=5e-4, seed=4, instances=inst, cell_occupancy=occupancy, device=device)
        configs.c2_network(s)
        s.finalize()
        s.set_ensemble_particles(pos, sp, counts)
        return s

    progress("batched: tuning on a scaled copy")
    tuned = tune.tune(lambda occ: build(mine[::8], occ), steps=20, warmup=5)
    progress("batched: timed run")
    steps = max(args.steps, 2000)
    s = build(mine, tuned["occupancy"])
    s.set_launch_shape(*tuned["shape"])
    s.step(args.warmup)
    s.synchronize()
    n0 = int(np.sum(s.instance_counts()))
    dist.barrier()
    ms = s.time_steps(steps)
    dist.barrier()
    n1 = int(np.sum(s.instance_counts()))
    prof = s.profile_steps(20)
    kms = {k: v / 20 for k, v in prof.items()}
    ms_max = dist.max(ms)
    batched = dist.sum(steps * 0.5 * (n0 + n1)) / (ms_max / 1e3)
    s.close()
    # the same instances advanced one after another as plain systems
    progress("batched: plain per-instance loop")
    loop_steps = 10
    total_ms = 0.0
    total_ps = 0.0
    for k in mine:
        inst, counts, pos, sp = share([k])
        p = configs.build_c2_instance(inst[0], int(counts[0]), device=device)
        p.set_particles(pos, sp)
        p.step(3)
        p.synchronize()
        total_ms += p.time_steps(loop_steps)
        total_ps += loop_steps * int(counts[0])
        p.close()
    loop = dist.sum(total_ps) / (dist.max(total_ms) / 1e3)
    return {"workload": f"c4: {len(inst_all)} instances of the c2 network, {int(np.sum(counts_all))} particles"
                        + (f", split over {dist.world} ranks by particle count" if dist.world > 1 else ""),
            "value": batched, "unit": UNIT, "steps": steps, "ms_per_step": ms_max / steps,
            "kernel_ms_per_step": kms, "launch_gaps_ms_per_step": ms / steps - sum(kms.values()),
            "tuned": {"cell_occupancy": tuned["occupancy"], "launch_shape": list(tuned["shape"]),
                      "tuning_s": round(tuned["tuning_s"], 2), "tuned_on": f"every 8th instance of the share "
                                                                           f"({len(mine[::8])} instances)"},
            "plain_loop_value": loop, "speedup_vs_plain_loop": batched / loop}


def run_serving(args, device):
    """c5: Poisson arrivals at 50/s of c3-network simulations with N
    log-uniform in 1e3-5e6 and steps uniform in 100-10000, admitted into one
    serving handle against a 150 GB budget; then the same requests served
    one at a time as plain systems (the baseline)."""
    from gpusmoldyn_gb300 import configs
    from gpusmoldyn_gb300.serve import Server, c3_request, run_sequential

    jobs = configs.c5_jobs(args.serve_jobs, seed=5)
    # each request arrives with its initial state (the client builds it)
    for j in jobs:
        j["payload"] = c3_request(j)
    srv = Server(max_instances=64, hbm_budget=150e9, chunk=10, device=device)
    res = srv.run(jobs)
    srv.close()
    progress("serving: one request at a time")
    seq = run_sequential(jobs, device=device)
    return {"workload": f"c5: {len(jobs)} requests, Poisson 50/s, N log-U[1e3, 5e6], steps U[100, 10000]",
            "p50_latency_s": res["p50_s"], "p99_latency_s": res["p99_s"], "mean_latency_s": res["mean_s"],
            "value": res["particle_steps_per_s"], "unit": UNIT, "wall_s": res["wall_s"], "jobs": res["jobs"],
            "seconds": {k: round(v, 4) for k, v in res["host_seconds"].items()},
            "one_at_a_time": {"p50_latency_s": seq["p50_s"], "p99_latency_s": seq["p99_s"],
                              "mean_latency_s": seq["mean_s"], "value": seq["particle_steps_per_s"],
                              "wall_s": seq["wall_s"]},
            "speedup_vs_one_at_a_time": res["particle_steps_per_s"] / seq["particle_steps_per_s"]}


def main():
    args = parse()
    dist = Dist(args.gpus)
    try:
        if args.impl == "reference":
            out = run_reference(args, dist)
        else:
            out = run_gb300(args, dist)
        if out is not None and dist.rank == 0:
            progress("done")
            print(json.dumps(out))
    finally:
        dist.close()


if __name__ == "__main__":
    main()
