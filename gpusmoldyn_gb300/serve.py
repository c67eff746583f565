"""Continuous-batching request loop over a serving handle.

Requests (simulations with their own size, seed and step count) arrive over
time.  Each loop iteration admits the requests that have arrived while a
slot and the HBM budget allow, advances every admitted simulation together
by a chunk of steps (one pipeline over all of them, one graph launch per
step), then harvests the simulations that reached their step count.  A
simulation freezes on the device at exactly its step count, so chunking
never overshoots, and it evolves bit for bit as it would alone.  It is
harvested one chunk after it freezes: by then a step has put its records
back in canonical order on the device, and the harvest is a device export.
"""
from __future__ import annotations

import collections
import math
import time

import numpy as np

from . import _lib as L
from .configs import c3_add_network, c3_network, c3_species, c3_steady_state, rng, uniform_positions
from .system import System

# device bytes per particle slot: two state buffers + the sort staging buffer
# (16 B each) + the matcher word (4 B), with 2x headroom for growth
BYTES_PER_PARTICLE = 2 * (16 * 3 + 4)


def c3_request(job, density=2.0):
    """Initial state of one c3-style request: n particles of the 8-species
    network at the c3 density in a cube sized for them."""
    n = job["n"]
    side = float((n / density) ** (1.0 / 3.0))
    desc = dict(box_lo=(0.0, 0.0, 0.0), box_hi=(side, side, side), seed=job["seed"])
    g = rng(job["seed"])
    pos = uniform_positions(g, n, desc["box_lo"], desc["box_hi"])
    _, frac = c3_steady_state(c3_network()[1], density)
    return desc, pos, c3_species(n, frac), job["steps"]


def c3_server_network(s, density=2.0, network_seed=3):
    c3_add_network(s, density, network_seed)
    s.finalize()


class Server:
    def __init__(self, network=c3_server_network, max_instances=64, hbm_budget=150e9, dt=1e-3, chunk=10,
                 device=0, normals="boxmuller"):
        self.s = System(dt=dt, instances=max_instances, device=device, normals=normals)
        network(self.s)
        self.max_instances = max_instances
        self.budget = hbm_budget
        self.chunk = chunk

    def run(self, jobs, make_request=c3_request, time_scale=1.0, keep_results=False):
        """Serve `jobs` (dicts with arrival [s], n, steps, seed); returns
        per-job latencies and throughput figures."""
        s = self.s
        pending = collections.deque(sorted(jobs, key=lambda j: j["arrival"]))
        waiting = collections.deque()
        active = {}  # slot -> (job, bytes)
        used = 0.0
        done = []
        seen = set()  # slots reported finished by the previous poll
        psteps = 0.0
        spent = collections.defaultdict(float)  # host seconds per activity
        t0 = time.perf_counter()
        while pending or waiting or active:
            now = time.perf_counter() - t0
            while pending and pending[0]["arrival"] * time_scale <= now:
                waiting.append(pending.popleft())
            while waiting and len(active) < self.max_instances:
                job = waiting[0]
                need = job["n"] * BYTES_PER_PARTICLE
                if used + need > self.budget and active:
                    break
                ta = time.perf_counter()
                desc, pos, sp, steps = job["payload"] if "payload" in job else make_request(job)
                tb = time.perf_counter()
                try:
                    slot = s.admit(desc, pos, sp, steps)
                except L.BDError as e:
                    # a slot harvested in this iteration is released by the
                    # next step: admit again after it
                    if e.code != L.BD_ERR_CAPACITY or not active:
                        raise
                    spent["admit"] += time.perf_counter() - tb
                    break
                waiting.popleft()
                spent["make_request"] += tb - ta
                spent["admit"] += time.perf_counter() - tb
                job["admitted"] = time.perf_counter() - t0
                active[slot] = (job, need)
                used += need
            if not active:
                if pending:
                    time.sleep(max(0.0, pending[0]["arrival"] * time_scale - (time.perf_counter() - t0)))
                continue
            live = sum(j["n"] for j, _ in active.values())
            ta = time.perf_counter()
            s.step(self.chunk)
            s.synchronize()
            tb = time.perf_counter()
            spent["steps"] += tb - ta
            psteps += live * self.chunk
            finished = s.poll()
            spent["poll"] += time.perf_counter() - tb
            ready = [slot for slot in finished if slot in seen]
            seen = set(finished) - set(ready)
            for slot in ready:
                job, need = active.pop(slot)
                tc = time.perf_counter()
                pos, sp = s.harvest(slot)
                spent["harvest"] += time.perf_counter() - tc
                job["finished"] = time.perf_counter() - t0
                job["latency"] = job["finished"] - job["arrival"] * time_scale
                job["n_final"] = int(len(sp))
                if keep_results:
                    job["result"] = (pos, sp)
                used -= need
                done.append(job)
        wall = time.perf_counter() - t0
        lat = np.array([j["latency"] for j in done])
        work = float(sum(j["n"] * j["steps"] for j in done))
        return dict(jobs=len(done), wall_s=wall, p50_s=float(np.percentile(lat, 50)),
                    p99_s=float(np.percentile(lat, 99)), mean_s=float(lat.mean()),
                    particle_steps_per_s=work / wall, approx_device_particle_steps=psteps, done=done,
                    host_seconds=dict(spent))

    def close(self):
        self.s.close()


def run_sequential(jobs, make_request=c3_request, device=0, dt=1e-3, normals="boxmuller", density=2.0):
    """The same requests served one at a time, in arrival order, on the wall
    clock: each waits for the previous one to finish, then runs alone as a
    plain system (handle, network, upload, its steps, readback) -- the
    baseline that continuous batching is measured against."""
    order = sorted(jobs, key=lambda j: j["arrival"])
    lat = []
    work = 0.0
    t0 = time.perf_counter()
    for job in order:
        now = time.perf_counter() - t0
        if job["arrival"] > now:
            time.sleep(job["arrival"] - now)
        desc, pos, sp, steps = job["payload"] if "payload" in job else make_request(job)
        s = System(desc["box_lo"], desc["box_hi"], dt=dt, seed=desc["seed"], normals=normals, device=device)
        c3_add_network(s, density)
        s.finalize()
        s.set_particles(pos, sp)
        s.step(steps)
        s.particles()
        s.close()
        lat.append(time.perf_counter() - t0 - job["arrival"])
        work += float(job["n"] * job["steps"])
    wall = time.perf_counter() - t0
    lat = np.array(lat)
    return dict(jobs=len(order), wall_s=wall, p50_s=float(np.percentile(lat, 50)),
                p99_s=float(np.percentile(lat, 99)), mean_s=float(lat.mean()), particle_steps_per_s=work / wall)
