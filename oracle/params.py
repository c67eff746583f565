"""The oracle's inputs derived without the library -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU leg use this module.

The library derives the step's inputs on the host: species diffusion
coefficients, reaction probabilities, binding radii, product offsets,
zeroth-order Poisson CDFs, the normal-quantile table and each instance's
uniform grid.  This module restates that derivation from the reference's
algorithms, in code of its own, so that

* the oracle can be set up from a network description alone -- bench.py's
  reference arm does this and never loads libgpusmoldyn.so -- and
* tests can compare the library's derivation with an independent one
  (tests/test_oracle_params.py).

Sources restated:
* numrxnrate / bindingradius / unbindingradius: the Andrews-Bray lookup
  (rxnparam.cpp:42-308; public domain, rxnparam.cpp:1-3), cubic Lagrange
  interpolation in ln(step/a) and in b/a or ln(b/a), with the reference's
  stencil rules and 15-step bisections, in the same floating-point
  operation order so that radii come out with the same bits;
* rxnsetrate (smolreact.cpp:283-397): order 0 -> Poisson mean k dt V,
  order 1 -> k/sum k (1 - exp(-dt sum k)) conditioned on the earlier
  reactions of the reactant, order 2 -> binding radius of rate k (2k for
  A + A);
* rxnsetproduct (smolreact.cpp:410-483): two products at +b D1/sum D and
  -b D2/sum D;
* the reversible coupling of the library (the binding radius calibrated
  with the unbinding radius b solved from the geminate probability; b = 0
  when the request is unattainable), the reference's intent that its code
  does not reach (smolreact.cpp:373-376, 459);
* poisrandF's distribution (stats.cpp:234-275) as an explicit CDF;
* createGaussTable's quantiles (stats.cpp:202-211);
* the grid rule: cells at least 1.01 x the largest binding radius, else
  sized for 3 records per cell (the reference's fixed 2 x particleRadius,
  particleSystem.cpp:69-76, is unrelated to the radius).

The rate tables themselves are read as data from the library's generated
header gpusmoldyn_gb300/csrc/rate_tables.h: its 868 values agree with the
reference's printed tables (rxnparam.cpp:43-157), which tests pin.
Transcendental functions come from the C library through ctypes, as the
library's host code calls them (numpy's float32 functions and CPython's own
lgamma need not round like them).
"""
from __future__ import annotations

import ctypes
import ctypes.util
import math
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TABLES_H = os.path.join(HERE, "..", "gpusmoldyn_gb300", "csrc", "rate_tables.h")

# product-placement kinds (the values of BD_PP_* in include/gpusmoldyn.h)
PP_DEFAULT, PP_PGEM, PP_PGEMMAX, PP_UNBINDRAD, PP_OFFSET0 = 0, 1, 2, 3, 4

_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
_libm.expf.restype = ctypes.c_float
_libm.expf.argtypes = [ctypes.c_float]
for _name in ("cbrt", "lgamma", "exp", "log", "erfc"):
    getattr(_libm, _name).restype = ctypes.c_double
    getattr(_libm, _name).argtypes = [ctypes.c_double]

f32 = np.float32


def expf(x):
    return f32(_libm.expf(float(x)))


# ------------------------------------------------------------ rate tables
_tables = None


def rate_tables():
    """(irreversible row, far rows, near rows, steps) from the header."""
    global _tables
    if _tables is None:
        txt = open(TABLES_H).read()
        dims = dict(re.findall(r"(k\w+) = (\d+)", txt.split("\n")[6]))

        def arr(name):
            body = re.search(name + r"\[[^\]]*\] = \{([^}]*)\}", txt).group(1)
            return np.array([float(v) for v in body.replace("\n", " ").split(",") if v.strip()])

        steps = int(dims["kSteps"])
        _tables = (arr("kIrrev"), arr("kRevFar").reshape(int(dims["kRowsR"]), steps),
                   arr("kRevNear").reshape(int(dims["kRowsB"]), steps), steps)
    return _tables


def _weights(s, nodes, h):
    # cubic Lagrange weights of 4 equally spaced nodes, denominators
    # multiplied left to right (rxnparam.cpp:174-177)
    x0, x1, x2, x3 = nodes
    return ((s - x1) * (s - x2) * (s - x3) / (-6.0 * h * h * h),
            (s - x0) * (s - x2) * (s - x3) / (2.0 * h * h * h),
            (s - x0) * (s - x1) * (s - x3) / (-2.0 * h * h * h),
            (s - x0) * (s - x1) * (s - x2) / (6.0 * h * h * h))


def numrxnrate(step, a, b):
    """Reactive flux per step (um^3) of a pair at binding radius a, rms step
    `step` and unbinding radius b (b < 0 irreversible)."""
    irrev, far, near, n_steps = rate_tables()
    S0, DS, BN0, DBN, BF0, DBF = 3.0, -0.2, 0.0, 0.1, 0.0, 0.2
    if step < 0 or a < 0:
        return -1.0
    if step == 0:
        return -1.0 if 0 <= b < 1 else 0.0
    ls = math.log(step / a)
    b = b / a
    col = int((ls - S0) / DS)

    def nodes(c, x0, h):
        return [x0 + (c - 1 + i) * h for i in range(4)]

    x = nodes(col, S0, DS)
    z = _weights(ls, x, DS)
    if b < 0:
        ans = 0.0
        for i in range(4):
            c = col - 1 + i
            if c >= n_steps:
                ans += z[i] * 2.0 * math.pi * math.exp(2.0 * x[i])
            elif c < 0:
                ans += z[i] * 4.0 * math.pi / 3.0
            else:
                ans += z[i] * irrev[c]
        return ans * a * a * a
    if b < 1.0:
        rows = near.shape[0]
        row = min(max(int((b - BN0) / DBN), 1), rows - 3)
        while col + 3 >= n_steps or (col > 0 and near[row - 1, col + 3] < 0):
            col -= 1
        x = nodes(col, S0, DS)
        z = _weights(ls, x, DS)
        y = []
        for j in range(4):
            acc = 0.0
            for i in range(4):
                c = col - 1 + i
                if c >= n_steps:
                    acc += z[i] * near[row - 1 + j, 0]
                elif c < 0:
                    acc += z[i] * 4.0 * math.pi / 3.0
                else:
                    acc += z[i] * near[row - 1 + j, c]
            y.append(acc)
        w = _weights(b, nodes(row, BN0, DBN), DBN)
    else:
        b = math.log(b)
        rows = far.shape[0]
        row = min(max(int((b - BF0) / DBF), 1), rows - 3)
        y = []
        for j in range(4):
            acc = 0.0
            for i in range(4):
                c = col - 1 + i
                if c >= n_steps and b == 0:
                    acc += z[i] * 2.0 * math.pi * math.exp(x[i]) * (1.0 + math.exp(x[i]))
                elif c >= n_steps:
                    acc += z[i] * 2.0 * math.pi * math.exp(2.0 * x[i]) * math.exp(b) / (math.exp(b) - 1.0)
                elif c < 0:
                    acc += z[i] * 4.0 * math.pi / 3.0
                else:
                    acc += z[i] * far[row - 1 + j, c]
            y.append(acc)
        w = _weights(b, nodes(row, BF0, DBF), DBF)
    ans = w[0] * y[0] + w[1] * y[1] + w[2] * y[2] + w[3] * y[3]
    return ans * a * a * a


def bindingradius(rate, dt, difc, b, rel):
    """Radius a with numrxnrate(step, a, b) = rate dt: doubling, then 15
    bisections (rxnparam.cpp:242-277)."""
    if rate < 0 or dt < 0 or difc <= 0:
        return -1.0
    if rate == 0:
        return 0.0
    if dt == 0:
        if b < 0:
            return rate / (4 * math.pi * difc)
        if rel and b > 1:
            return rate * (1 - 1 / b) / (4 * math.pi * difc)
        if rel:
            return -1.0
        return rate / (4 * math.pi * difc + rate / b) if b > 0 else -1.0
    step = math.sqrt(2.0 * difc * dt)
    target = rate * dt
    lo, a = 0.0, step
    while numrxnrate(step, a, b * a if rel else b) < target:
        lo, a = a, a * 2.0
    dif = a - lo
    for _ in range(15):
        dif *= 0.5
        a = lo + dif
        if numrxnrate(step, a, b * a if rel else b) < target:
            lo = a
    return lo + 0.5 * dif


def unbindingradius(pgem, dt, difc, a):
    """Unbinding radius b giving geminate probability pgem; -2 for illegal
    input, -pgem_max when pgem is above the maximum (rxnparam.cpp:280-308)."""
    if pgem <= 0 or pgem >= 1 or difc <= 0 or a <= 0 or dt < 0:
        return -2.0
    if dt == 0:
        return a / pgem
    step = math.sqrt(2.0 * difc * dt)
    ki, kmax = numrxnrate(step, a, -1), numrxnrate(step, a, 0)
    if 1.0 - ki / kmax < pgem:
        return ki / kmax - 1.0
    lo, b = 0.0, a
    while 1.0 - ki / numrxnrate(step, a, b) > pgem:
        lo, b = b, b * 2.0
    dif = b - lo
    for _ in range(15):
        dif *= 0.5
        b = lo + dif
        if 1.0 - ki / numrxnrate(step, a, b) > pgem:
            lo = b
    return lo + 0.5 * dif


# --------------------------------------------------------- distributions
def poisson_cdf(mean):
    """CDF of Poisson(mean) over [kmin, kmin + len): all but ~1e-30 of the
    mass, the last entry forced to 1.  Returns (cdf, kmin)."""
    if not mean > 0:
        return np.ones(1), 0
    sd = math.sqrt(mean)
    lo = max(0, int(math.floor(mean - 12.0 * sd - 10.0)))
    hi = int(math.ceil(mean + 12.0 * sd + 10.0))
    lm = _libm.log(mean)
    out = np.empty(hi - lo + 1)
    acc = 0.0
    for k in range(lo, hi + 1):
        acc += _libm.exp(-mean + k * lm - _libm.lgamma(k + 1.0))
        out[k - lo] = min(acc, 1.0)
    out[-1] = 1.0
    return out, lo


def gauss_quantiles(n=4096):
    """Standard-normal quantiles at (i + 1/2) / n, by bisection on the normal
    CDF in double precision, antisymmetric (createGaussTable's values)."""
    out = np.zeros(n, np.float32)
    for i in range(n // 2):
        p = (i + 0.5) / n
        lo, hi = -40.0, 0.0
        for _ in range(200):
            if not hi - lo > 0:
                break
            mid = 0.5 * (lo + hi)
            if mid == lo or mid == hi:
                break
            if 0.5 * _libm.erfc(-mid / math.sqrt(2.0)) < p:
                lo = mid
            else:
                hi = mid
        out[i] = f32(0.5 * (lo + hi))
        out[n - 1 - i] = -out[i]
    return out


# -------------------------------------------------------------- reactions
class Reaction:
    """One reaction as a caller gives it: order, reactants, products, rate,
    product placement kind and parameter, per-encounter probability (order
    2; < 0 = 1)."""

    def __init__(self, order, reactants, products, rate, pp_kind=PP_DEFAULT, pp_param=0.0, user_prob=-1.0):
        self.order = order
        self.reactants = list(reactants) + [-1] * (2 - len(reactants))
        self.products = list(products) + [-1] * (2 - len(products))
        self.nprod = len(products)
        self.rate = f32(rate)
        self.pp_kind = pp_kind
        self.pp_param = f32(pp_param)
        self.user_prob = f32(user_prob)


def _same_pair(a, b):
    return sorted(a) == sorted(b)


def reverse_of(rx, r):
    """The reaction that undoes r (findreverserxn, smolreact.cpp:73-146)."""
    f = rx[r]
    if f.order == 0 or f.nprod < 1:
        return -1
    for q, g in enumerate(rx):
        if q == r or g.order != f.nprod or g.nprod != f.order:
            continue
        rct = g.reactants[0] == f.products[0] if g.order == 1 else _same_pair(g.reactants, f.products)
        prd = g.products[0] == f.reactants[0] if f.order == 1 else _same_pair(g.products, f.reactants)
        if rct and prd:
            return q
    return -1


def derive(D0, rx, dt, volume, d_scale=1.0, k2_scale=1.0):
    """Per-species D and per-reaction inputs of one parameter block (the
    last listed reaction of a species pair is its reaction; competing
    channels are not restated here).  Float quantities are rounded to
    float32 at every operation, as the library computes them."""
    dt, volume, d_scale, k2_scale = f32(dt), f32(volume), f32(d_scale), f32(k2_scale)
    S, R = len(D0), len(rx)
    D = np.array([f32(d) * d_scale for d in D0], np.float32)
    out = dict(D=D, prob=np.zeros(R, np.float32), bind_radius=np.zeros(R, np.float32),
               unbind_radius=np.zeros(R, np.float32), off0=np.zeros(R, np.float32), off1=np.zeros(R, np.float32),
               flags=np.zeros(R, np.int32), cdf=[np.zeros(0)] * R, cdf_kmin=[0] * R, status=0)
    rev = [reverse_of(rx, r) for r in range(R)]

    def fail(code):
        if out["status"] == 0:
            out["status"] = code

    for r, q in enumerate(rx):
        if q.order == 0:
            if q.rate < 0:
                fail(1)
                continue
            out["prob"][r] = q.rate * dt * volume
            out["cdf"][r], out["cdf_kmin"][r] = poisson_cdf(float(out["prob"][r]))
    for r, q in enumerate(rx):
        if q.order != 1:
            continue
        if q.rate < 0:
            fail(1)
            continue
        sp = q.reactants[0]
        total = f32(0)
        for g in rx:
            if g.order == 1 and g.reactants[0] == sp and g.rate > 0:
                total = f32(total + g.rate)
        if q.rate == 0:
            continue
        p = f32(0)
        if total > 0:
            p = q.rate / total * (f32(1) - expf(-dt * total))
        prior = f32(0)
        for g in range(r):
            if rx[g].order == 1 and rx[g].reactants[0] == sp:
                prior = f32(prior + out["prob"][g])
        out["prob"][r] = p / (f32(1) - prior)
    for r, q in enumerate(rx):
        if q.order != 2:
            continue
        out["prob"][r] = q.user_prob if q.user_prob >= 0 else f32(1)
        i1, i2 = q.reactants
        if q.rate < 0:
            fail(1)
            continue
        rate3 = f32(q.rate * k2_scale)
        if i1 == i2:
            rate3 = f32(rate3 * f32(2))
        dsum = f32(D[i1] + D[i2])
        if rate3 <= 0:
            continue
        if dsum <= 0:
            fail(4)
            continue
        rate3, dtd, dsd = float(rate3), float(dt), float(dsum)
        u = rev[r]
        if u >= 0 and rx[u].order == 1 and rx[u].nprod == 2:
            kind, p = rx[u].pp_kind, float(rx[u].pp_param)
            if kind == PP_DEFAULT:
                kind, p = PP_PGEMMAX, 0.2
            b = 0.0
            step = math.sqrt(2.0 * dsd * dtd)
            if kind == PP_UNBINDRAD:
                b = p
                a = bindingradius(rate3, dtd, dsd, b, 0)
            elif kind == PP_OFFSET0:
                a = bindingradius(rate3, dtd, dsd, 0, 0)
            else:
                a0 = bindingradius(rate3, dtd, dsd, 0, 0)
                pmax = 1.0 - numrxnrate(step, a0, -1) / numrxnrate(step, a0, 0)
                if not 0 < p < 1:
                    fail(7)
                    a = a0
                elif p >= pmax:
                    if kind == PP_PGEM:
                        fail(8)
                    a = a0
                    out["flags"][u] |= 1
                else:
                    a = a0
                    for _ in range(200):
                        b = unbindingradius(p, dtd, dsd, a)
                        if b < 0:
                            break
                        an = bindingradius(rate3, dtd, dsd, b, 0)
                        done = abs(an - a) <= 1e-9 * a
                        a = an
                        if done:
                            break
                    if b < 0:
                        fail(8)
                        b, a = 0.0, a0
                        out["flags"][u] |= 1
            out["unbind_radius"][u] = f32(b)
        else:
            a = bindingradius(rate3, dtd, dsd, -1, 0)
        out["bind_radius"][r] = f32(a)
    for r, q in enumerate(rx):
        if q.nprod != 2:
            continue
        dc1, dc2 = D[q.products[0]], D[q.products[1]]
        dsum = f32(dc1 + dc2)
        b = out["unbind_radius"][r]
        coupled = rev[r] >= 0 and rx[rev[r]].order == 2 and q.order == 1
        if not coupled:
            b = q.pp_param if q.pp_kind == PP_UNBINDRAD else f32(0)
            out["unbind_radius"][r] = b
            if dsum == 0:
                dc1, dc2, dsum = f32(1), f32(1), f32(0.5)
        elif dsum <= 0:
            fail(4)
            continue
        out["off0"][r] = b * dc1 / dsum
        out["off1"][r] = -b * dc2 / dsum
    return out


# -------------------------------------------------------------------- grid
def plan_grid(box_lo, box_hi, n_particles, r_max, occupancy=3.0, cell_size=0.0):
    """Cells per axis, cell edges and cells per unit length (float32) of
    one instance: at least 1.01 x the largest binding radius, otherwise
    about `occupancy` records per cell, at most 2^28 cells."""
    L = [float(f32(box_hi[a])) - float(f32(box_lo[a])) for a in range(3)]
    vol = 1.0
    for v in L:
        vol *= v
    if cell_size > 0:
        cs = float(f32(cell_size))
    else:
        cs = _libm.cbrt(occupancy * vol / float(max(int(n_particles), 1)))
    cs = max(cs, 1.01 * float(f32(r_max)))
    for _ in range(64):
        total = 1
        for v in L:
            total *= int(max(1.0, math.floor(v / cs)))
        if total <= (1 << 28):
            break
        cs *= 1.25
    dims = np.array([int(max(1.0, math.floor(v / cs))) for v in L], np.uint32)
    cell = np.array([f32(L[a] / float(dims[a])) for a in range(3)], np.float32)
    inv = np.array([f32(dims[a]) / f32(L[a]) for a in range(3)], np.float32)
    return dims, cell, inv
