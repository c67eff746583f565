"""Autotuner for the step: cell occupancy (cell edge) and launch shapes.

The cell edge trades the cost of the sort (histogram and cell-start words
per cell, atomics per cell per warp) against the in-cell work of the pair
kernel (canonical ranks are O(occupancy) per particle).  Launch shapes
trade occupancy against scheduling overhead.  Candidates are timed with
CUDA events on a scaled copy of the workload (same density, fewer
particles), which transfers because the optimum depends on the density and
the network, not on N.

The cell edge changes the canonical order and hence the random streams, so
a tuned configuration is a reproducible choice recorded with the results
rather than an invisible optimisation; the launch shape does not change
results at all.
"""
from __future__ import annotations

import time


def time_config(build, occupancy, shape, steps=20, warmup=5):
    s = build(occupancy)
    if shape:
        s.set_launch_shape(*shape)
    s.step(warmup)
    s.synchronize()
    n = s.count()
    ms = s.time_steps(steps)
    s.close()
    return ms / steps, n


def tune(build, occupancies=(1.5, 2.0, 3.0, 4.0, 6.0, 8.0),
         shapes=((256, 4, 256, 4), (256, 8, 256, 4), (128, 8, 256, 4), (256, 4, 256, 8), (256, 4, 256, 16)),
         steps=20, warmup=5):
    """`build(occupancy)` returns a System with particles set.  Returns the
    best (occupancy, shape) and the timing table."""
    t0 = time.perf_counter()
    table = []
    best_occ, best = None, None
    for occ in occupancies:
        ms, n = time_config(build, occ, shapes[0], steps, warmup)
        table.append(dict(occupancy=occ, shape=shapes[0], ms_per_step=ms, particles=n))
        if best is None or ms < best:
            best, best_occ = ms, occ
    best_shape = shapes[0]
    for shape in shapes[1:]:
        ms, n = time_config(build, best_occ, shape, steps, warmup)
        table.append(dict(occupancy=best_occ, shape=shape, ms_per_step=ms, particles=n))
        if ms < best:
            best, best_shape = ms, shape
    return dict(occupancy=best_occ, shape=best_shape, ms_per_step=best, table=table,
                tuning_s=time.perf_counter() - t0)
