"""Generator for the bimolecular reaction-rate tables used by ``numrxnrate``.

The tables hold the steady-state reactive flux of the Andrews-Bray algorithm
(S. S. Andrews and D. Bray, "Stochastic simulation of chemical reactions with
spatial resolution and single molecule detail", Phys. Biol. 1:137-151, 2004):
a pair of molecules diffuses with rms step ``s`` (in units of the binding
radius ``a``), reacts whenever it ends a step closer than ``a``, and (for a
reversible reaction) is put back at separation ``b`` after it reacts.  The
radial distribution function (RDF) of the pair is advanced by alternating a
diffusion step (convolution with the radial Green's function) and an
absorption step (everything inside ``r < 1`` is removed and counted as flux)
until the flux per step stops changing.  The flux at steady state, in units of
``a**3``, is the reaction rate times the time step.

This module restates that published numerical method in matrix form: one
diffusion step plus one absorption step is an affine map ``x -> M x + c`` of
the sampled RDF, so each (s, b) point builds ``M`` once in O(n^2) and then
iterates matrix-vector products.  The discretisation follows the one the
reference's tables were produced with (rxnparam.cpp:329-477, rdfabsorb /
rdfdiffuse / rdfreverserxn / rdfsteadystate; grid and sweep parameters
rxnparam.cpp:484-559): a uniform radial grid starting at 0 whose first point
at or above 1 is replaced by the pair 0.9999 / 1.0001, the spherical
trapezoid rule for both integrals, a ``1 + a2/r`` fit of the last 10% of the
grid for the tail beyond the grid, the fractional-change stopping rule with
at least 30 and at most 100000 iterations, and warm starts along the sweep
in step length.  The three tables are:

* ``yi``: irreversible reactions, 31 step lengths ln(s) = 3, 2.8, ..., -3,
  600 radial points, eps 1e-5; the mean of an increasing and a decreasing sweep
  (the reference lists these as "600 pts, eps=1e-5, up&down").
* ``yr``: reversible with b > a, ln(b) = 0, 0.2, ..., 3 (16 rows), 500 points,
  mean of both sweeps.
* ``yb``: reversible with b <= a, b = 0, 0.1, ..., 1 (11 rows), 100 points,
  decreasing sweep only; an entry whose iteration diverges is stored as -1.

Run ``python -m gpusmoldyn_gb300.rate_tables_gen`` to rewrite
``csrc/rate_tables.h``; the header is committed so the library build needs no
numerical work.  Runtime is a few minutes on one core.
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

SQRT2PI = math.sqrt(2.0 * math.pi)
MAXIT = 100000
MAXFLUX = 1e7


def radial_grid(n: int, dr: float) -> np.ndarray:
    """Uniform grid from 0 whose first point >= 1 becomes 0.9999, followed by 1.0001."""
    r = [0.0]
    while r[-1] < 1.0 and len(r) <= n:
        r.append(r[-1] + dr)
    r[-1] = 0.9999
    r.append(1.0001)
    while len(r) < n:
        r.append(r[-1] + dr)
    return np.asarray(r[:n], dtype=np.float64)


def _seg_weights(r0, r1):
    """Spherical trapezoid weights (for f0, f1) of one segment [r0, r1].

    With f linear between (r0, f0) and (r1, f1), the shell integral
    int 4 pi r^2 f dr equals f0 * w0 + f1 * w1."""
    p = math.pi * (r1 + r0) * (r1 * r1 + r0 * r0)
    q = 4.0 * math.pi / 3.0 * (r1 * r1 + r1 * r0 + r0 * r0)
    return -p + q * r1, p - q * r0


def _node_weights(t: np.ndarray) -> np.ndarray:
    """Trapezoid weights for a chain of nodes t[0..m-1] (first node at t=0)."""
    m = len(t)
    w = np.zeros(m)
    for k in range(1, m):
        w0, w1 = _seg_weights(t[k - 1], t[k])
        w[k - 1] += w0
        w[k] += w1
    return w


def _erfc(x):
    return np.vectorize(math.erfc)(x)


def diffusion_map(r: np.ndarray, step: float):
    """Affine map (A, c) of one diffusion step: rdf_out = A @ rdf_in + c."""
    n = len(r)
    A = np.zeros((n, n))
    c = np.zeros(n)
    start = int(0.9 * n)
    alpha = np.sum(1.0 / r[start:] ** 2)
    # a2 = sum_{m>=start} (rdf[m]-1)/r[m] / alpha / step  (tail fit rdf ~ 1 + a2/r)
    a2_row = np.zeros(n)
    a2_row[start:] = 1.0 / r[start:] / alpha / step
    a2_const = -np.sum(a2_row)

    zero_first = r[0] == 0.0
    jlist = np.arange(1, n) if zero_first else np.arange(0, n)
    tj = r[jlist] / step
    # node chain: virtual node at t=0 (value index 0) followed by the grid nodes
    tnodes = np.concatenate(([0.0], tj))
    idx = np.concatenate(([0], jlist))
    w = _node_weights(tnodes)
    tlast = tnodes[-1]

    i0 = 0
    if zero_first:
        g0 = np.exp(-tnodes ** 2 / 2.0) / (2.0 * math.pi * SQRT2PI)
        wg = w * g0
        wg[0] = 0.0  # the node at t=0 carries rdf[0]-rdf[0] = 0
        np.add.at(A[0], idx, wg)
        A[0, 0] -= wg.sum()
        tail = 4.0 * math.pi * tlast * g0[-1] + math.erfc(tlast / math.sqrt(2.0))
        A[0, 0] += 1.0 - tail
        c[0] += tail
        i0 = 1

    rows = np.arange(i0, n)
    rr = r[rows] / step
    # Green's function of radial diffusion, rows x nodes
    t = tnodes[None, :]
    with np.errstate(divide="ignore", invalid="ignore"):
        G = (np.exp(-(rr[:, None] - t) ** 2 / 2.0) - np.exp(-(rr[:, None] + t) ** 2 / 2.0)) / (
            rr[:, None] * t) / (4.0 * math.pi * SQRT2PI)
    G[:, 0] = np.exp(-rr ** 2 / 2.0) / (2.0 * math.pi * SQRT2PI)
    WG = G * w[None, :]
    for k, row in enumerate(rows):
        np.add.at(A[row], idx, WG[k])
    A[rows, rows] -= WG.sum(axis=1)
    erfcdif = _erfc((tlast - rr) / math.sqrt(2.0))
    erfcsum = _erfc((tlast + rr) / math.sqrt(2.0))
    tail = 4.0 * math.pi * tlast * G[:, -1] + 0.5 * (erfcdif + erfcsum)
    A[rows, rows] += 1.0 - tail
    c[rows] += tail
    U = 0.5 / rr * (erfcdif - erfcsum)
    A[rows, :] += U[:, None] * a2_row[None, :]
    c[rows] += U * a2_const
    return A, c


def absorption(r: np.ndarray):
    """Linear flux functional and the count of leading points set to zero."""
    n = len(r)
    wa = np.zeros(n)
    r1 = 0.0
    i1 = 0
    j = 1 if r[0] == 0.0 else 0
    r0 = 0.0
    while r1 < 1.0 and j < n:
        r0, i0 = r1, i1
        r1, i1 = r[j], j
        w0, w1 = _seg_weights(r0, r1)
        wa[i0] += w0
        wa[i1] += w1
        j += 1
    # the last segment keeps only the part carried by its inner point
    wa[i1] -= _seg_weights(r0, r1)[1]
    nzero = max(j - 1, 0)
    return wa, nzero


def reverse_kernel(r: np.ndarray, step: float, b: float) -> np.ndarray:
    """RDF added per unit flux re-injected at separation b, after one step."""
    k = 1.0 / (4.0 * math.pi * SQRT2PI * step ** 3)
    rr = r / step
    g = np.zeros(len(r))
    if b == 0.0:
        return 2.0 * k * np.exp(-rr ** 2 / 2.0)
    bs = b / step
    i0 = 0
    if r[0] == 0.0:
        g[0] = 2.0 * k * math.exp(-bs * bs / 2.0)
        i0 = 1
    q = rr[i0:]
    g[i0:] = k / q / bs * (np.exp(-(q - bs) ** 2 / 2.0) - np.exp(-(q + bs) ** 2 / 2.0))
    return g


def steady_flux(r, x, step, b, eps):
    """Alternate diffusion and absorption from the RDF ``x`` (updated in place)
    until the flux settles; returns the flux or -1 on divergence."""
    A, c = diffusion_map(r, step)
    wa, nzero = absorption(r)
    g = reverse_kernel(r, step, b) if b >= 0 else None
    y = A @ x + c
    flux = fluxold = float(wa @ y)
    it = 0
    while it < 30 or (it < MAXIT and flux < MAXFLUX and
                      abs((flux - fluxold) / (fluxold + 1e-20)) > eps):
        fluxold = flux
        y = A @ x + c
        if g is not None:
            y = y + flux * g
        x[:] = y
        flux = float(wa @ x)
        x[:nzero] = 0.0
        it += 1
    if it >= MAXIT or flux >= MAXFLUX or not math.isfinite(flux):
        return -1.0
    return flux


def initial_rdf(r, mode, up, b):
    """Trial RDF: 0 up to the first grid point >= 1, then the analytic
    irreversible / reversible profile (increasing sweeps) or 1."""
    n = len(r)
    x = np.zeros(n)
    i = 0
    while i < n and r[i] < 1.0:
        i += 1
    if up and mode == "i":
        x[i:] = 1.0 - 1.0 / r[i:]
        return x
    if up and mode == "r":
        while i < n and r[i] < b:
            x[i] = 1.0 - (b - r[i]) / r[i] / (b - 1.0)
            i += 1
    x[i:] = 1.0
    return x


def sweep(mode, n, eps, up, b=-1.0):
    """Flux at ln(s) = 3, 2.8, ..., -3 (table order) for one sweep direction."""
    logs = [-3.0 + 0.2 * k for k in range(31)]
    if not up:
        logs = logs[::-1]
    if mode == "i":
        dr = 10.0 / n
    elif mode == "r":
        dr = (b + 3.0) / n
    else:
        dr = 5.0 / n
    r = radial_grid(n, dr)
    x = initial_rdf(r, mode, up, b)
    out = {}
    flux = 0.0
    for ls in logs:
        if flux >= 0:
            flux = steady_flux(r, x, math.exp(ls), b, eps)
        out[round(ls, 6)] = flux
    return [out[round(3.0 - 0.2 * k, 6)] for k in range(31)]


def _round6(v):
    """Six decimals, as the sweeps are tabulated; diverged points stay -1."""
    return -1.0 if v < 0 else float("%.6f" % v)


def _mean6(up, dn):
    """Mean of the two sweeps, each rounded to six decimals first."""
    out = []
    for u, d in zip(up, dn):
        out.append(-1.0 if (u < 0 or d < 0) else 0.5 * (_round6(u) + _round6(d)))
    return out


def build_tables(verbose=False):
    def log(msg):
        if verbose:
            print(msg, file=sys.stderr, flush=True)

    up = sweep("i", 600, 1e-5, True)
    dn = sweep("i", 600, 1e-5, False)
    yi = _mean6(up, dn)
    log("yi done")
    yr = []
    for k in range(16):
        b = math.exp(0.2 * k)
        up = sweep("r", 500, 1e-5, True, b)
        dn = sweep("r", 500, 1e-5, False, b)
        yr += _mean6(up, dn)
        log(f"yr row {k} done")
    yb = []
    for k in range(11):
        b = 0.1 * k
        yb += [_round6(v) for v in sweep("b", 100, 1e-5, False, b)]
        log(f"yb row {k} done")
    return yi, yr, yb


def _fmt(vals):
    out = []
    for k in range(0, len(vals), 8):
        out.append("  " + ", ".join(("%.7f" % v) if v >= 0 else "-1" for v in vals[k:k + 8]) + ",")
    return "\n".join(out)


def write_header(path, yi, yr, yb):
    with open(path, "w") as f:
        f.write("// Generated by gpusmoldyn_gb300/rate_tables_gen.py: steady-state reactive flux\n")
        f.write("// per time step (units of a^3) of the Andrews-Bray algorithm, rows of 31 step\n")
        f.write("// lengths ln(s/a) = 3, 2.8, ..., -3.  -1 marks a diverged steady state.\n")
        f.write("#pragma once\n\nnamespace bd_tables {\n")
        f.write("static const int kSteps = 31, kRowsR = 16, kRowsB = 11;\n")
        f.write("static const double kIrrev[31] = {\n%s\n};\n" % _fmt(yi))
        f.write("static const double kRevFar[16 * 31] = {\n%s\n};\n" % _fmt(yr))
        f.write("static const double kRevNear[11 * 31] = {\n%s\n};\n" % _fmt(yb))
        f.write("}  // namespace bd_tables\n")


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    yi, yr, yb = build_tables(verbose=True)
    write_header(os.path.join(here, "csrc", "rate_tables.h"), yi, yr, yb)


if __name__ == "__main__":
    main()
