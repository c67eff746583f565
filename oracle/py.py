"""ctypes wrapper of liboracle.so -- TEST INFRASTRUCTURE, not product.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module.  ``OracleSystem(sys)`` reads a configured library handle's
parameters through the public C ABI (species D, reaction table entries,
grid, Poisson CDFs, normal table) and turns them into the oracle's inputs;
``OracleSystem.from_network`` derives them instead with ``oracle.params``
from a network description alone, without loading the library.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

fp = C.POINTER(C.c_float)
ip = C.POINTER(C.c_int)
dp = C.POINTER(C.c_double)


class or_system(C.Structure):
    _fields_ = [("lo", C.c_float * 3), ("hi", C.c_float * 3), ("inv", C.c_float * 3), ("cell", C.c_float * 3),
                ("dims", C.c_uint32 * 3), ("key_lo", C.c_uint32), ("key_hi", C.c_uint32),
                ("normal_mode", C.c_int), ("gauss", fp), ("S", C.c_int), ("D", fp), ("dt", C.c_float),
                ("R", C.c_int), ("order", ip), ("react0", ip), ("react1", ip), ("prod0", ip), ("prod1", ip),
                ("prob", fp), ("bind_radius", fp), ("off0", fp), ("off1", fp), ("cdf", dp), ("cdf_off", ip),
                ("cdf_len", ip), ("cdf_kmin", ip), ("sorted", C.c_int), ("inst", C.c_uint32),
                ("threads", C.c_int), ("channels", C.c_int), ("thresh", fp), ("n_panels", C.c_int),
                ("panels", C.c_void_p), ("surf_act", C.c_void_p)]


_lib = None


def load():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        lib = C.CDLL(path)
        lib.or_step.restype = C.c_int
        lib.or_step.argtypes = [C.POINTER(or_system), C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32,
                                C.POINTER(C.c_uint32), C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint32,
                                C.POINTER(C.c_uint32), C.c_void_p]
        lib.or_philox.restype = None
        lib.or_philox.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]
        _lib = lib
    return _lib


def philox(ctr, k0, k1):
    lib = load()
    c = np.asarray(ctr, np.uint32)
    out = np.zeros(4, np.uint32)
    lib.or_philox(c.ctypes.data, k0, k1, out.ctypes.data)
    return out


class OracleSystem:
    """Oracle inputs for one instance of a library handle."""

    def __init__(self, sys, instance=0, threads=0, sorted_path=None):
        from gpusmoldyn_gb300 import _lib as L
        from gpusmoldyn_gb300.system import gauss_table

        self.keep = []
        d = sys.instances[instance]
        dims, cell, inv = sys.grid(instance)
        D = sys.species_d(instance)
        R = sys.n_reactions
        info = [sys.reaction_info(r, instance) for r in range(R)]
        order = np.array([i["order"] for i in info] or [0], np.int32)
        react0 = np.array([i["reactants"][0] for i in info] or [0], np.int32)
        react1 = np.array([i["reactants"][1] for i in info] or [0], np.int32)
        prod0 = np.array([i["products"][0] for i in info] or [0], np.int32)
        prod1 = np.array([i["products"][1] for i in info] or [0], np.int32)
        prob = np.array([i["prob"] for i in info] or [0], np.float32)
        brad = np.array([i["bind_radius"] for i in info] or [0], np.float32)
        off0 = np.array([i["product_offsets"][0] for i in info] or [0], np.float32)
        off1 = np.array([i["product_offsets"][1] for i in info] or [0], np.float32)
        thresh = np.array([i["channel_threshold"] for i in info] or [1], np.float32)
        cdfs, coff, clen, ckmin = [], [], [], []
        pos = 0
        for r in range(R):
            if info[r]["order"] == 0:
                cdf, kmin = sys.poisson_cdf(r, instance)
            else:
                cdf, kmin = np.zeros(0), 0
            cdfs.append(cdf)
            coff.append(pos)
            clen.append(len(cdf))
            ckmin.append(kmin)
            pos += len(cdf)
        cdf_all = np.concatenate(cdfs) if pos else np.zeros(1)
        gauss = gauss_table()
        self._fill(order, react0, react1, prod0, prod1, prob, brad, off0, off1, thresh, D, gauss, cdf_all, coff,
                   clen, ckmin)
        arrs = self.arrs
        s = self._system(d["box_lo"], d["box_hi"], dims, cell, inv, int(d.get("seed", 1)), sys.cfg.normal_mode,
                         sys.n_species, sys.dt, R)
        # surfaces: the panels' derived geometry (bd_panel_info words) and the
        # [surface][species][front, back] action table, read through the C ABI
        n_surf, n_pan = sys.surface_counts()
        pan = np.zeros((max(n_pan, 1), 23), np.uint32)
        for k in range(n_pan):
            q = L.bd_panel_info()
            L.check(sys.lib.bd_get_panel(sys.h, k, C.byref(q)), "bd_get_panel")
            pan[k] = np.frombuffer(bytes(q), np.uint32)
        act = np.zeros(max(n_surf * sys.n_species * 2, 1), np.uint8)
        for f in range(n_surf):
            for sp in range(sys.n_species):
                for face in (0, 1):
                    act[(f * sys.n_species + sp) * 2 + face] = sys.surface_action(f, sp, face)
        arrs["panels"] = pan
        arrs["surf_act"] = act
        s.n_panels = n_pan
        s.panels = pan.ctypes.data
        s.surf_act = act.ctypes.data
        if sorted_path is None:
            sorted_path = (sys.n_instances > 1 or any(i["order"] in (1, 2) for i in info)
                           or any(i["order"] == 0 and i["nprod"] == 2 for i in info) or n_pan > 0)
        s.sorted = 1 if sorted_path else 0
        s.inst = instance
        s.threads = threads
        s.channels = 1 if getattr(sys.cfg, "pair_mode", 0) == 1 else 0
        self.s = s
        self.n_cells = int(dims[0]) * int(dims[1]) * int(dims[2])
        self.R = R

    def _fill(self, order, react0, react1, prod0, prod1, prob, brad, off0, off1, thresh, D, gauss, cdf_all, coff,
              clen, ckmin):
        self.keep = []
        self.arrs = dict(order=order, react0=react0, react1=react1, prod0=prod0, prod1=prod1, prob=prob,
                         bind_radius=brad, off0=off0, off1=off1, thresh=thresh, D=np.asarray(D, np.float32),
                         gauss=gauss, cdf=np.asarray(cdf_all, np.float64), cdf_off=np.array(coff or [0], np.int32),
                         cdf_len=np.array(clen or [0], np.int32), cdf_kmin=np.array(ckmin or [0], np.int32))

    def _system(self, lo, hi, dims, cell, inv, seed, normal_mode, S, dt, R):
        arrs = self.arrs
        s = or_system()
        for a in range(3):
            s.lo[a] = lo[a]
            s.hi[a] = hi[a]
            s.inv[a] = inv[a]
            s.cell[a] = cell[a]
            s.dims[a] = int(dims[a])
        s.key_lo = seed & 0xFFFFFFFF
        s.key_hi = seed >> 32
        s.normal_mode = normal_mode
        s.S = S
        s.dt = dt
        s.R = R
        for name in ("order", "react0", "react1", "prod0", "prod1", "cdf_off", "cdf_len", "cdf_kmin"):
            setattr(s, name, arrs[name].ctypes.data_as(ip))
        for name in ("prob", "bind_radius", "off0", "off1", "thresh", "D", "gauss"):
            setattr(s, name, arrs[name].ctypes.data_as(fp))
        s.cdf = arrs["cdf"].ctypes.data_as(dp)
        return s

    @classmethod
    def from_network(cls, D, reactions, box_lo, box_hi, dt, seed, n_particles, normal_mode=0, threads=0,
                     d_scale=1.0, k2_scale=1.0, occupancy=3.0, cell_size=0.0):
        """An oracle whose inputs are derived by oracle.params from a network
        description: D per species and a list of oracle.params.Reaction.  The
        grid is planned for n_particles; no library is loaded."""
        from . import params as P

        self = cls.__new__(cls)
        R = len(reactions)
        vol = np.float32(np.float32(box_hi[0] - box_lo[0]) * np.float32(box_hi[1] - box_lo[1])) \
            * np.float32(box_hi[2] - box_lo[2])
        der = P.derive(D, reactions, dt, vol, d_scale, k2_scale)
        if der["status"]:
            raise RuntimeError(f"oracle.params: set-up error {der['status']}")
        r_max = max([float(der["bind_radius"][r]) for r in range(R) if reactions[r].order == 2] or [0.0])
        dims, cell, inv = P.plan_grid(box_lo, box_hi, n_particles, r_max, occupancy, cell_size)
        col = lambda f, dt_: np.array([f(q) for q in reactions] or [0], dt_)  # noqa: E731
        cdfs, coff, clen, ckmin, pos = [], [], [], [], 0
        for r in range(R):
            c = der["cdf"][r] if reactions[r].order == 0 else np.zeros(0)
            cdfs.append(c)
            coff.append(pos)
            clen.append(len(c))
            ckmin.append(der["cdf_kmin"][r] if reactions[r].order == 0 else 0)
            pos += len(c)
        gauss = P.gauss_quantiles() if normal_mode == 1 else np.zeros(4096, np.float32)
        self._fill(col(lambda q: q.order, np.int32), col(lambda q: q.reactants[0], np.int32),
                   col(lambda q: q.reactants[1], np.int32), col(lambda q: q.products[0], np.int32),
                   col(lambda q: q.products[1], np.int32), der["prob"] if R else np.zeros(1, np.float32),
                   der["bind_radius"] if R else np.zeros(1, np.float32), der["off0"] if R else np.zeros(1, np.float32),
                   der["off1"] if R else np.zeros(1, np.float32), np.ones(max(R, 1), np.float32), der["D"], gauss,
                   np.concatenate(cdfs) if pos else np.zeros(1), coff, clen, ckmin)
        s = self._system(box_lo, box_hi, dims, cell, inv, int(seed), normal_mode, len(D), dt, R)
        s.n_panels = 0
        s.panels = None
        s.surf_act = None
        s.sorted = 1 if any(q.order in (1, 2) or (q.order == 0 and q.nprod == 2) for q in reactions) else 0
        s.inst = 0
        s.threads = threads
        s.channels = 0
        self.s = s
        self.n_cells = int(dims[0]) * int(dims[1]) * int(dims[2])
        self.R = R
        self.grid = (dims, cell, inv)
        self.derived = der
        return self

    def step(self, t, recs, want_cells=False, want_pairs=False, cap=None, events=None):
        """Advance records (n x 4 uint32: x, y, z bits and w) by one step."""
        lib = load()
        recs = np.ascontiguousarray(recs, np.uint32)
        n = recs.shape[0]
        cap = cap or max(4 * n + 1024, 4096)
        out = np.zeros((cap, 4), np.uint32)
        n_out = C.c_uint32()
        cells = np.zeros(self.n_cells + 1, np.uint32) if want_cells else None
        pcap = 1 << 22
        pairs = np.zeros((pcap, 4), np.uint32) if want_pairs else None
        n_pairs = C.c_uint32()
        ev = events if events is not None else np.zeros(max(self.R, 1), np.uint64)
        rc = lib.or_step(C.byref(self.s), t, recs.ctypes.data if n else None, n, out.ctypes.data, cap,
                         C.byref(n_out), cells.ctypes.data if cells is not None else None,
                         self.n_cells + 1, pairs.ctypes.data if pairs is not None else None, pcap,
                         C.byref(n_pairs), ev.ctypes.data)
        if rc != 0:
            raise RuntimeError(f"oracle step failed ({rc})")
        res = dict(recs=out[:n_out.value].copy(), events=ev)
        if want_cells:
            res["cells"] = cells
        if want_pairs:
            res["pairs"] = pairs[:n_pairs.value].copy()
        return res


def records(pos, species, inst=0):
    """Pack (n,3) float32 positions and species into oracle records."""
    pos = np.asarray(pos, np.float32)
    n = pos.shape[0]
    r = np.zeros((n, 4), np.uint32)
    r[:, :3] = pos[:, :3].view(np.uint32)
    r[:, 3] = (np.uint32(inst) << np.uint32(16)) | np.asarray(species, np.uint32)
    return r


def slots_to_records(xyz, w):
    r = np.zeros((xyz.shape[0], 4), np.uint32)
    r[:, :3] = np.ascontiguousarray(xyz, np.float32).view(np.uint32)
    r[:, 3] = w
    dead = w == 0xFFFFFFFF
    r[dead, :3] = 0
    return r


def default_threads():
    return int(os.environ.get("ORACLE_THREADS", "0"))
