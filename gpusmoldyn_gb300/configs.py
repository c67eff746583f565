"""Seeded synthetic systems with the shapes of the benchmark configurations.

No public dataset is involved: initial positions are drawn uniformly in the
box from numpy's Philox generator with the configuration's seed.

* c1: irreversible A + B -> C, 20k + 20k in a 10 um cube, D 1/1/0.5, k 0.01,
  dt 1 ms (the reference-scale CPU-runnable case).
* c2: reversible A + B <-> C, 500k + 500k in a 60 um cube, k_on 0.05,
  k_off 10, dt 0.5 ms.
* c3: 8-species network, 16M particles in a 200 um cube, 12 reactions
  (2 zeroth, 4 first, 5 hetero- and 1 homodimeric second order), D log-uniform
  0.1-10, rates log-uniform over a decade, dt 1 ms, started at the network's
  stationary composition so the particle count stays put.
* c4: 256 instances of the c2 network, N log-uniform 1e3-1e6 (about 37M),
  per-instance D and k_on scaled log-uniform over a decade, c2 density.
* c5: serving jobs, c3 network, N log-uniform 1e3-5e6, steps U[100, 10000],
  Poisson arrivals at 50/s.
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib as L
from .system import System


def rng(seed):
    return np.random.Generator(np.random.Philox(seed))


def uniform_positions(g, n, lo, hi):
    lo = np.asarray(lo, np.float32)
    hi = np.asarray(hi, np.float32)
    p = lo + (hi - lo) * g.random((n, 3), dtype=np.float32)
    return np.minimum(np.maximum(p, lo), hi).astype(np.float32)


# ---------------------------------------------------------------- c1 / c2
def build_c1(n_a=20000, n_b=20000, side=10.0, seed=1, normals="boxmuller", **kw):
    s = System((0, 0, 0), (side, side, side), dt=1e-3, seed=seed, normals=normals, **kw)
    A, B, Cc = s.add_species(1.0), s.add_species(1.0), s.add_species(0.5)
    s.add_reaction(2, [A, B], [Cc], 0.01)
    s.finalize()
    g = rng(seed)
    pos = uniform_positions(g, n_a + n_b, (0, 0, 0), (side, side, side))
    sp = np.concatenate([np.full(n_a, A), np.full(n_b, B)]).astype(np.int32)
    s.set_particles(pos, sp)
    return s


def c2_network(s, kon=0.05, koff=10.0):
    A, B, Cc = s.add_species(1.0), s.add_species(1.0), s.add_species(0.5)
    fwd = s.add_reaction(2, [A, B], [Cc], kon)
    back = s.add_reaction(1, [Cc], [A, B], koff)
    s.set_product_placement(back, L.BD_PP_PGEMMAX, 0.2)
    return A, B, Cc, fwd, back


def c2_system(side=60.0, seed=2, normals="boxmuller", **kw):
    s = System((0, 0, 0), (side, side, side), dt=5e-4, seed=seed, normals=normals, **kw)
    c2_network(s)
    s.finalize()
    return s


def c2_particles(n_a=500000, n_b=500000, side=60.0, seed=2):
    g = rng(seed)
    pos = uniform_positions(g, n_a + n_b, (0, 0, 0), (side, side, side))
    sp = np.concatenate([np.zeros(n_a), np.ones(n_b)]).astype(np.int32)
    return pos, sp


def build_c2(n_a=500000, n_b=500000, side=60.0, seed=2, normals="boxmuller", **kw):
    s = c2_system(side, seed, normals, **kw)
    s.set_particles(*c2_particles(n_a, n_b, side, seed))
    return s


# ---------------------------------------------------------------------- c3
def c3_network(seed=3):
    """Species diffusion coefficients and the 10 non-zeroth reactions (order,
    reactants, products, rate) of the 8-species network.

    S0 and S1 are made by the two zeroth-order reactions; S4/S5 and S6/S7
    are carrier pairs whose totals are conserved; S3 -> 0 is the only exit.
    Every species is made and consumed, so the network has one stable
    stationary composition (c3_steady_state) and a run started there keeps
    its particle count.  Rates are log-uniform over one decade: first order
    0.01-0.1 /s, second order 0.01-0.1 um^3/s."""
    g = rng(seed)
    D = np.exp(g.uniform(math.log(0.1), math.log(10.0), 8)).astype(np.float32)
    k1 = np.exp(g.uniform(math.log(0.01), math.log(0.1), 4))
    k2 = np.exp(g.uniform(math.log(0.01), math.log(0.1), 6))
    rx = [
        (2, [0, 1], [2], k2[0]),      # S0 + S1 -> S2
        (1, [2], [3], k1[0]),         # S2 -> S3
        (2, [3, 4], [5], k2[1]),      # S3 + S4 -> S5
        (1, [5], [4], k1[1]),         # S5 -> S4
        (2, [0, 6], [7], k2[2]),      # S0 + S6 -> S7
        (2, [1, 6], [7], k2[3]),      # S1 + S6 -> S7
        (1, [7], [6], k1[2]),         # S7 -> S6
        (2, [2, 4], [5], k2[4]),      # S2 + S4 -> S5
        (2, [2, 2], [3], k2[5]),      # S2 + S2 -> S3
        (1, [3], [], k1[3]),          # S3 -> 0
    ]
    return D, rx


def _mass_action(rho, z, rx):
    """d rho / dt of the well-mixed network; a homodimeric A + A reaction of
    rate k fires k rho_A^2 times per unit volume and time (its binding
    radius is computed for rate 2k)."""
    d = np.zeros(len(rho))
    d[0] += z
    d[1] += z
    for order, rc, pr, k in rx:
        r = k * rho[rc[0]] if order == 1 else k * rho[rc[0]] * rho[rc[1]]
        for a in rc:
            d[a] -= r
        for b in pr:
            d[b] += r
    return d


def c3_steady_state(rx, density):
    """Zeroth-order rate z (per unit volume and time, each of S0 and S1) and
    species fractions of the stationary well-mixed state with total density
    `density`, each carrier pair holding a quarter of it.  Newton's method
    on the 6 independent rate equations, the 2 carrier totals and the total."""
    quarter = density / 4.0

    def F(x):
        rho, z = x[:8], x[8]
        d = _mass_action(rho, z, rx)
        return np.array([d[0], d[1], d[2], d[3], d[4], d[6], rho[4] + rho[5] - quarter,
                         rho[6] + rho[7] - quarter, rho.sum() - density])

    x = np.full(9, density / 8.0)
    x[8] = 1e-3 * density
    for _ in range(100):
        f = F(x)
        if np.max(np.abs(f)) < 1e-13 * density:
            break
        J = np.empty((9, 9))
        for j in range(9):
            e = np.zeros(9)
            e[j] = 1e-7 * max(abs(x[j]), 1e-6)
            J[:, j] = (F(x + e) - f) / e[j]
        dx = np.linalg.solve(J, -f)
        t = 1.0
        while np.any(x + t * dx <= 0):
            t *= 0.5
        x = x + t * dx
    else:
        raise RuntimeError("c3 steady state did not converge")
    return float(x[8]), x[:8] / density


def c3_species(n, frac):
    """n species ids with the stationary fractions (largest remainders)."""
    want = np.asarray(frac) * n
    cnt = np.floor(want).astype(np.int64)
    rest = n - int(cnt.sum())
    cnt[np.argsort(-(want - cnt))[:rest]] += 1
    return np.repeat(np.arange(len(frac), dtype=np.int32), cnt)


def c3_reactions(density, network_seed=3):
    """Diffusion coefficients, the 12 reactions (order, reactants, products,
    rate) in the order they are added -- the two zeroth-order productions
    first -- and the stationary species fractions of the c3 network at
    `density`."""
    D, rx = c3_network(network_seed)
    z, frac = c3_steady_state(rx, density)
    return D, [(0, [], [0], z), (0, [], [1], z)] + [(o, rc, pr, float(k)) for o, rc, pr, k in rx], frac


def c3_add_network(s, density, network_seed=3):
    """Species and the 12 reactions of the c3 network on a System; returns
    the stationary species fractions."""
    D, rx, frac = c3_reactions(density, network_seed)
    for d in D:
        s.add_species(float(d))
    for order, rc, pr, k in rx:
        s.add_reaction(order, rc, pr, k)
    return frac


def icosphere(centre, radius, levels):
    """Triangles (k, 3, 3) of an icosahedron subdivided `levels` times and
    pushed onto the sphere, vertices counterclockwise seen from outside."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    V = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    tris = np.array([[V[a], V[b], V[c]] for a, b, c in F], np.float64)
    tris /= np.linalg.norm(tris, axis=2, keepdims=True)
    for _ in range(levels):
        a, b, c = tris[:, 0], tris[:, 1], tris[:, 2]
        ab, bc, ca = (a + b) / 2, (b + c) / 2, (c + a) / 2
        tris = np.concatenate([np.stack(q, 1) for q in ((a, ab, ca), (ab, b, bc), (ca, bc, c), (ab, bc, ca))])
        tris /= np.linalg.norm(tris, axis=2, keepdims=True)
    return np.asarray(centre, np.float64) + radius * tris


def c3_cell_surfaces(s, side):
    """The c3 network inside a cell: a spherical membrane (radius 0.4 side)
    that reflects every species but the two small ligands S0 and S1, which
    cross it, and a nucleus (radius 0.12 side, an icosphere of 1280
    triangles) that reflects every species.  Nothing is absorbed, so the
    stationary composition of the plain c3 run is kept."""
    c = (side / 2, side / 2, side / 2)
    membrane = s.add_surface()
    s.set_surface_action(membrane, -1, "both", "reflect")
    for lig in (0, 1):
        s.set_surface_action(membrane, lig, "both", "transmit")
    s.add_panel(membrane, "sph", [c[0], c[1], c[2], 0.4 * side])
    nucleus = s.add_surface()
    s.set_surface_action(nucleus, -1, "both", "reflect")
    for tri in icosphere(c, 0.12 * side, 3):
        s.add_panel(nucleus, "tri", list(tri.ravel()))


def c3_system(n=16_000_000, side=200.0, seed=3, normals="boxmuller", network_seed=3, surfaces=False, **kw):
    """The c3 network in a `side` cube, finalized, without particles
    (surfaces: inside the cell of c3_cell_surfaces)."""
    s = System((0, 0, 0), (side, side, side), dt=1e-3, seed=seed, normals=normals, **kw)
    c3_add_network(s, n / side ** 3, network_seed)
    if surfaces:
        c3_cell_surfaces(s, side)
    s.finalize()
    return s


def c3_particles(n=16_000_000, side=200.0, seed=3, network_seed=3):
    """n particles, uniform in the cube, at the stationary composition."""
    g = rng(seed)
    pos = uniform_positions(g, n, (0, 0, 0), (side, side, side))
    _, rx = c3_network(network_seed)
    _, frac = c3_steady_state(rx, n / side ** 3)
    return pos, c3_species(n, frac)


def build_c3(n=16_000_000, side=200.0, seed=3, normals="boxmuller", network_seed=3, surfaces=False, **kw):
    s = c3_system(n, side, seed, normals, network_seed, surfaces, **kw)
    s.set_particles(*c3_particles(n, side, seed, network_seed))
    return s


# ---------------------------------------------------------------------- c4
C2_DENSITY = 1_000_000 / 60.0 ** 3


def c4_instances(n_inst=256, seed=4, n_lo=1e3, n_hi=1e6):
    g = rng(seed)
    counts = np.exp(g.uniform(math.log(n_lo), math.log(n_hi), n_inst)).astype(np.int64)
    counts += counts % 2  # even: half A, half B
    dsc = np.exp(g.uniform(math.log(10 ** -0.5), math.log(10 ** 0.5), n_inst))
    ksc = np.exp(g.uniform(math.log(10 ** -0.5), math.log(10 ** 0.5), n_inst))
    inst = []
    for k in range(n_inst):
        side = float((counts[k] / C2_DENSITY) ** (1.0 / 3.0))
        inst.append(dict(box_lo=(0.0, 0.0, 0.0), box_hi=(side, side, side), seed=1000 + k,
                         d_scale=float(dsc[k]), k2_scale=float(ksc[k])))
    return inst, counts


def c4_positions(inst, counts, seed=4):
    g = rng(seed + 1)
    pos, sp = [], []
    for d, n in zip(inst, counts):
        pos.append(uniform_positions(g, int(n), d["box_lo"], d["box_hi"]))
        sp.append(np.concatenate([np.zeros(n // 2, np.int32), np.ones(n - n // 2, np.int32)]))
    return np.concatenate(pos), np.concatenate(sp)


def build_c4(n_inst=256, seed=4, normals="boxmuller", n_lo=1e3, n_hi=1e6, **kw):
    inst, counts = c4_instances(n_inst, seed, n_lo, n_hi)
    s = System(dt=5e-4, seed=seed, normals=normals, instances=inst, **kw)
    c2_network(s)
    s.finalize()
    pos, sp = c4_positions(inst, counts, seed)
    s.set_ensemble_particles(pos, sp, counts)
    return s, inst, counts


def build_c2_instance(d, n, seed=4, normals="boxmuller", **kw):
    """One c4 instance alone, as a single system with the same parameters."""
    s = System(dt=5e-4, seed=seed, normals=normals, instances=[d], **kw)
    c2_network(s)
    s.finalize()
    return s


# ---------------------------------------------------------------------- c5
def c5_jobs(n_jobs, seed=5, rate_hz=50.0, n_lo=1e3, n_hi=5e6, steps_lo=100, steps_hi=10000):
    g = rng(seed)
    arrivals = np.cumsum(g.exponential(1.0 / rate_hz, n_jobs))
    ns = np.exp(g.uniform(math.log(n_lo), math.log(n_hi), n_jobs)).astype(np.int64)
    steps = g.integers(steps_lo, steps_hi + 1, n_jobs)
    return [dict(id=k, arrival=float(arrivals[k]), n=int(ns[k]), steps=int(steps[k]), seed=5000 + k)
            for k in range(n_jobs)]
