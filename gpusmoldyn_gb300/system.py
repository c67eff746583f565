"""Pythonic handle over the C ABI: one simulation or one batched ensemble."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class System:
    """One Brownian-dynamics simulation (or ensemble) resident on one GPU.

    ``instances`` (list of dicts with box_lo, box_hi, seed, d_scale, k2_scale,
    cell_size) makes an ensemble of independent instances sharing the
    species and reaction network.  ``sort`` picks how records reach their
    cells ("auto", "compact" or "binned"; identical results); ``pairs``
    whether several second-order reactions of one reactant pair compete
    ("channels") or the last listed one is the pair's reaction ("last")."""

    def __init__(self, box_lo=(0.0, 0.0, 0.0), box_hi=(1.0, 1.0, 1.0), dt=1e-3, seed=1, normals="boxmuller",
                 capacity=0, cell_size=0.0, cell_occupancy=0.0, pair_capacity=0, device=0, instances=None,
                 sort="auto", pairs="last"):
        self.lib = L.load()
        self.server = False
        cfg = L.bd_config()
        self.lib.bd_config_default(C.byref(cfg))
        for a in range(3):
            cfg.box_lo[a] = box_lo[a]
            cfg.box_hi[a] = box_hi[a]
        cfg.dt = dt
        cfg.seed = seed
        cfg.capacity = int(capacity)
        cfg.cell_size = cell_size
        cfg.cell_occupancy = cell_occupancy
        cfg.pair_capacity = int(pair_capacity)
        cfg.device = device
        cfg.normal_mode = L.BD_NORMALS_TABLE if normals == "table" else L.BD_NORMALS_BOXMULLER
        cfg.sort_mode = {"auto": L.BD_SORT_AUTO, "compact": L.BD_SORT_COMPACT, "binned": L.BD_SORT_BINNED}[sort]
        cfg.pair_mode = {"last": L.BD_PAIR_LAST, "channels": L.BD_PAIR_CHANNELS}[pairs]
        self.cfg = cfg
        self.dt = dt
        self.h = C.c_void_p()
        if isinstance(instances, int):
            # serving handle with `instances` slots filled by admit()
            L.check(self.lib.bd_create_server(C.byref(cfg), instances, C.byref(self.h)), "bd_create_server")
            self.server = True
            self.n_instances = instances
            self.instances = [dict(box_lo=tuple(box_lo), box_hi=tuple(box_hi), seed=seed + k, d_scale=1.0,
                                   k2_scale=1.0, cell_size=0.0) for k in range(instances)]
        elif instances is None:
            L.check(self.lib.bd_create(C.byref(cfg), C.byref(self.h)), "bd_create")
            self.n_instances = 1
            self.instances = [dict(box_lo=tuple(box_lo), box_hi=tuple(box_hi), seed=seed, d_scale=1.0,
                                   k2_scale=1.0, cell_size=0.0)]
        else:
            arr = (L.bd_instance_desc * len(instances))()
            for k, d in enumerate(instances):
                for a in range(3):
                    arr[k].box_lo[a] = d["box_lo"][a]
                    arr[k].box_hi[a] = d["box_hi"][a]
                arr[k].seed = d.get("seed", k + 1)
                arr[k].d_scale = d.get("d_scale", 1.0)
                arr[k].k2_scale = d.get("k2_scale", 1.0)
                arr[k].cell_size = d.get("cell_size", 0.0)
            L.check(self.lib.bd_create_ensemble(C.byref(cfg), arr, len(instances), C.byref(self.h)),
                    "bd_create_ensemble")
            self.n_instances = len(instances)
            self.instances = [dict(d) for d in instances]
        self.n_species = 0
        self.n_reactions = 0

    @classmethod
    def from_model(cls, text=None, path=None, device=0):
        """A finalized system with its molecules placed, from a model in the
        Smoldyn-style configuration language (bd_create_from_model).  Returns
        (system, info) with info the time span and counts the model declared."""
        self = cls.__new__(cls)
        self.lib = L.load()
        self.server = False
        self.h = C.c_void_p()
        info = L.bd_model_info()
        err = C.create_string_buffer(512)
        dev = L.BD_DEVICE_NONE if device is None else device
        if path is not None:
            rc = self.lib.bd_create_from_model_file(str(path).encode(), dev, C.byref(self.h), C.byref(info), err, 512)
        else:
            rc = self.lib.bd_create_from_model(text.encode(), dev, C.byref(self.h), C.byref(info), err, 512)
        if rc != L.BD_OK:
            raise L.BDError(rc, f"model: {err.value.decode()}")
        cfg = L.bd_config()
        L.check(self.lib.bd_get_config(self.h, C.byref(cfg)), "bd_get_config")
        self.cfg = cfg
        self.dt = cfg.dt
        self.n_instances = 1
        self.instances = [dict(box_lo=tuple(cfg.box_lo), box_hi=tuple(cfg.box_hi), seed=cfg.seed, d_scale=1.0,
                               k2_scale=1.0, cell_size=0.0)]
        self.n_species = info.n_species
        self.n_reactions = info.n_reactions
        return self, dict(time_start=info.time_start, time_stop=info.time_stop, steps=info.steps,
                          n_molecules=info.n_molecules)

    def species_id(self, name: str) -> int:
        i = C.c_int()
        L.check(self.lib.bd_find_species(self.h, name.encode(), C.byref(i)), f"species {name}")
        return i.value

    def reaction_id(self, name: str) -> int:
        i = C.c_int()
        L.check(self.lib.bd_find_reaction(self.h, name.encode(), C.byref(i)), f"reaction {name}")
        return i.value

    # ------------------------------------------------------------- set-up
    def add_species(self, D: float) -> int:
        i = C.c_int()
        L.check(self.lib.bd_add_species(self.h, D, C.byref(i)), "bd_add_species")
        self.n_species += 1
        return i.value

    def add_reaction(self, order, reactants=(), products=(), rate=0.0) -> int:
        r = (C.c_int * 2)(*(list(reactants) + [-1, -1])[:2])
        p = (C.c_int * 2)(*(list(products) + [-1, -1])[:2])
        i = C.c_int()
        L.check(self.lib.bd_add_reaction(self.h, order, r, p, rate, C.byref(i)), "bd_add_reaction")
        self.n_reactions += 1
        return i.value

    def set_product_placement(self, rxn, kind, param=0.0):
        L.check(self.lib.bd_set_product_placement(self.h, rxn, kind, param), "bd_set_product_placement")

    def set_reaction_probability(self, rxn, prob):
        L.check(self.lib.bd_set_reaction_probability(self.h, rxn, prob), "bd_set_reaction_probability")

    # surfaces
    _FACES = {"front": L.BD_FACE_FRONT, "back": L.BD_FACE_BACK, "both": L.BD_FACE_BOTH}
    _ACTIONS = {"transmit": L.BD_SURF_TRANSMIT, "reflect": L.BD_SURF_REFLECT, "absorb": L.BD_SURF_ABSORB}
    _SHAPES = {"rect": L.BD_PANEL_RECT, "tri": L.BD_PANEL_TRI, "sph": L.BD_PANEL_SPH, "cyl": L.BD_PANEL_CYL,
               "hemi": L.BD_PANEL_HEMI, "disk": L.BD_PANEL_DISK}

    def add_surface(self) -> int:
        i = C.c_int()
        L.check(self.lib.bd_add_surface(self.h, C.byref(i)), "bd_add_surface")
        return i.value

    def set_surface_action(self, surface, species=L.BD_ALL_SPECIES, face="both", action="reflect"):
        """species: id or BD_ALL_SPECIES; face and action by name or BD_* code."""
        face = self._FACES.get(face, face)
        action = self._ACTIONS.get(action, action)
        L.check(self.lib.bd_set_surface_action(self.h, surface, species, face, action), "bd_set_surface_action")

    def surface_action(self, surface, species, face) -> int:
        v = C.c_int()
        L.check(self.lib.bd_get_surface_action(self.h, surface, species, self._FACES.get(face, face), C.byref(v)),
                "bd_get_surface_action")
        return v.value

    def add_panel(self, surface, shape, params, axis=0, front=1) -> int:
        """One panel of `surface`: shape by name or BD_PANEL_* code, params as
        in bd_panel.p (rect: corner, two sides; tri: 3 vertices; sph: centre,
        radius; cyl: two ends, radius; hemi: centre, radius, opening
        direction; disk: centre, radius, normal)."""
        pn = L.bd_panel()
        pn.shape = self._SHAPES.get(shape, shape)
        pn.axis = axis
        pn.front = front
        vals = list(params)
        if len(vals) > 10:
            raise ValueError("at most 10 panel parameters")
        for k, v in enumerate(vals):
            pn.p[k] = v
        i = C.c_int()
        L.check(self.lib.bd_add_panel(self.h, surface, C.byref(pn), C.byref(i)), "bd_add_panel")
        return i.value

    def panel_info(self, pid) -> dict:
        q = L.bd_panel_info()
        L.check(self.lib.bd_get_panel(self.h, pid, C.byref(q)), "bd_get_panel")
        return {name: (list(getattr(q, name)) if hasattr(getattr(q, name), "__len__") else getattr(q, name))
                for name, _ in L.bd_panel_info._fields_}

    def surface_counts(self):
        ns, npn = C.c_int(), C.c_int()
        L.check(self.lib.bd_get_surface_counts(self.h, C.byref(ns), C.byref(npn)), "bd_get_surface_counts")
        return ns.value, npn.value

    def finalize(self, allow=(L.BD_OK, L.BD_ERR_PGEM_UNATTAINABLE)):
        st = self.lib.bd_finalize(self.h)
        L.check(st, "bd_finalize", ok=allow)
        return st

    def reaction_info(self, rxn, instance=0) -> dict:
        ri = L.bd_reaction_info()
        L.check(self.lib.bd_get_instance_reaction_info(self.h, instance, rxn, C.byref(ri)), "reaction_info")
        return dict(order=ri.order, nprod=ri.nprod, reactants=list(ri.reactants), products=list(ri.products),
                    rate=ri.rate, prob=ri.prob, bind_radius=ri.bind_radius, unbind_radius=ri.unbind_radius,
                    geminate_prob=ri.geminate_prob, product_offsets=list(ri.product_offsets),
                    reverse=ri.reverse, flags=ri.flags, channel_threshold=ri.channel_threshold)

    def species_d(self, instance=0) -> np.ndarray:
        out = np.zeros(self.n_species, np.float32)
        for s in range(self.n_species):
            v = C.c_float()
            L.check(self.lib.bd_get_species_d(self.h, instance, s, C.byref(v)), "species_d")
            out[s] = v.value
        return out

    def poisson_cdf(self, rxn, instance=0):
        kmin = C.c_int()
        n = C.c_size_t()
        L.check(self.lib.bd_get_poisson_cdf(self.h, instance, rxn, None, 0, C.byref(kmin), C.byref(n)), "cdf")
        buf = np.zeros(n.value, np.float64)
        L.check(self.lib.bd_get_poisson_cdf(self.h, instance, rxn, _ptr(buf), n.value, C.byref(kmin),
                                            C.byref(n)), "cdf")
        return buf, kmin.value

    # ---------------------------------------------------------- particles
    def set_particles(self, pos, species):
        """pos: (n, 3) or (n, 4) positions (a contiguous float32 (n, 4) array,
        the reference's float4 layout, is passed without a copy)."""
        pos = np.asarray(pos, np.float32)
        n = pos.shape[0]
        if pos.ndim == 2 and pos.shape[1] == 4 and pos.flags.c_contiguous:
            p4 = pos
        else:
            p4 = np.empty((n, 4), np.float32)
            p4[:, :3] = pos[:, :3]
            p4[:, 3] = 0.0
        sp = np.ascontiguousarray(species, np.int32)
        L.check(self.lib.bd_set_particles(self.h, _ptr(p4), _ptr(sp), n), "bd_set_particles")

    def set_ensemble_particles(self, pos, species, counts):
        pos = np.asarray(pos, np.float32)
        n = pos.shape[0]
        p4 = np.zeros((n, 4), np.float32)
        p4[:, :3] = pos[:, :3]
        sp = np.ascontiguousarray(species, np.int32)
        cnt = np.ascontiguousarray(counts, np.uint64)
        L.check(self.lib.bd_set_ensemble_particles(self.h, _ptr(p4), _ptr(sp), _ptr(cnt), len(cnt)),
                "bd_set_ensemble_particles")

    def step(self, n=1, stream=None):
        """Enqueue n steps; with `stream` (a cudaStream_t as an int) they are
        ordered after that stream's work and before its later work."""
        if stream is None:
            L.check(self.lib.bd_step(self.h, int(n)), "bd_step")
        else:
            L.check(self.lib.bd_step_async(self.h, int(n), C.c_void_p(stream)), "bd_step_async")

    def synchronize(self, allow_empty=True):
        st = self.lib.bd_synchronize(self.h)
        L.check(st, "bd_synchronize", ok=(L.BD_OK, L.BD_ERR_EMPTY) if allow_empty else (L.BD_OK,))
        return st

    def count(self) -> int:
        v = C.c_uint64()
        L.check(self.lib.bd_get_count(self.h, C.byref(v)), "bd_get_count")
        return v.value

    def step_count(self) -> int:
        v = C.c_uint64()
        L.check(self.lib.bd_get_step(self.h, C.byref(v)), "bd_get_step")
        return v.value

    def particles4(self, instance=-1, out=None):
        """Live particles in slot order as the reference's layout: (n, 4)
        float32 positions (w = 1) and int32 species.  out = (pos, species)
        arrays the caller keeps between calls (contiguous float32 (cap, 4)
        and int32 (cap,)) are filled instead of new ones; the views returned
        hold the first n."""
        n = self.count() if instance < 0 else int(self.instance_counts()[instance])
        if out is not None:
            pos, sp = out
            if (pos.dtype != np.float32 or sp.dtype != np.int32 or pos.ndim != 2 or pos.shape[1] != 4
                    or not pos.flags.c_contiguous or not sp.flags.c_contiguous or len(pos) < n or len(sp) < n):
                raise ValueError("out: contiguous float32 (>= n, 4) and int32 (>= n,) arrays")
        else:
            pos = np.empty((max(n, 1), 4), np.float32)
            sp = np.empty(max(n, 1), np.int32)
        got = C.c_size_t()
        L.check(self.lib.bd_get_instance_particles(self.h, instance, _ptr(pos), _ptr(sp), n, C.byref(got)),
                "bd_get_particles")
        m = min(got.value, n)
        return pos[:m], sp[:m]

    def particles(self, instance=-1):
        pos, sp = self.particles4(instance)
        return np.ascontiguousarray(pos[:, :3]), sp

    def species_counts(self, instance=-1) -> np.ndarray:
        out = np.zeros(max(self.n_species, 1), np.uint64)
        L.check(self.lib.bd_get_species_counts(self.h, instance, _ptr(out), self.n_species), "species_counts")
        return out[:self.n_species]

    def measure_msd(self, nsteps, instance=-1):
        """Take nsteps steps and return (msd, counts) per species: the mean
        squared diffusion move per step (bd_measure_msd)."""
        msd = np.zeros(max(self.n_species, 1), np.float64)
        cnt = np.zeros(max(self.n_species, 1), np.uint64)
        L.check(self.lib.bd_measure_msd(self.h, instance, int(nsteps), _ptr(msd), _ptr(cnt), self.n_species),
                "bd_measure_msd")
        return msd[:self.n_species], cnt[:self.n_species]

    def instance_counts(self) -> np.ndarray:
        out = np.zeros(self.n_instances, np.uint64)
        L.check(self.lib.bd_get_instance_counts(self.h, _ptr(out), self.n_instances), "instance_counts")
        return out

    def slots(self):
        n = C.c_size_t()
        L.check(self.lib.bd_debug_get_slots(self.h, None, None, 0, C.byref(n)), "slots")
        xyz = np.zeros((max(n.value, 1), 4), np.float32)
        w = np.zeros(max(n.value, 1), np.uint32)
        L.check(self.lib.bd_debug_get_slots(self.h, _ptr(xyz), _ptr(w), n.value, C.byref(n)), "slots")
        return xyz[:n.value, :3].copy(), w[:n.value].copy()

    def cells(self) -> np.ndarray:
        n = C.c_size_t()
        L.check(self.lib.bd_debug_get_cells(self.h, None, 0, C.byref(n)), "cells")
        out = np.zeros(n.value + 1, np.uint32)
        L.check(self.lib.bd_debug_get_cells(self.h, _ptr(out), n.value + 1, C.byref(n)), "cells")
        return out

    def pairs(self) -> np.ndarray:
        n = C.c_size_t()
        L.check(self.lib.bd_debug_get_pairs(self.h, None, 0, C.byref(n)), "pairs")
        out = np.zeros((max(n.value, 1), 4), np.uint32)
        L.check(self.lib.bd_debug_get_pairs(self.h, _ptr(out), n.value, C.byref(n)), "pairs")
        return out[:n.value].copy()

    def grid(self, instance=0):
        dims = np.zeros(3, np.uint32)
        cell = np.zeros(3, np.float32)
        inv = np.zeros(3, np.float32)
        L.check(self.lib.bd_get_grid(self.h, instance, _ptr(dims), _ptr(cell), _ptr(inv)), "bd_get_grid")
        return dims, cell, inv

    def event_counts(self) -> np.ndarray:
        out = np.zeros(max(self.n_reactions, 1), np.uint64)
        L.check(self.lib.bd_get_event_counts(self.h, _ptr(out), self.n_reactions), "event_counts")
        return out[:self.n_reactions]

    # ------------------------------------------------------------ serving
    def admit(self, desc, pos, species, steps) -> int:
        """Add a simulation to a serving handle; returns its slot."""
        d = L.bd_instance_desc()
        for a in range(3):
            d.box_lo[a] = desc["box_lo"][a]
            d.box_hi[a] = desc["box_hi"][a]
        d.seed = desc.get("seed", 1)
        d.d_scale = desc.get("d_scale", 1.0)
        d.k2_scale = desc.get("k2_scale", 1.0)
        d.cell_size = desc.get("cell_size", 0.0)
        pos = np.asarray(pos, np.float32)
        n = pos.shape[0]
        p4 = np.zeros((max(n, 1), 4), np.float32)
        p4[:n, :3] = pos[:, :3]
        sp = np.ascontiguousarray(species, np.int32)
        slot = C.c_int()
        L.check(self.lib.bd_instance_admit(self.h, C.byref(d), _ptr(p4), _ptr(sp), n, int(steps), C.byref(slot)),
                "bd_instance_admit")
        self.instances[slot.value] = dict(desc)
        return slot.value

    def poll(self):
        buf = np.zeros(max(self.n_instances, 1), np.int32)
        m = C.c_int()
        L.check(self.lib.bd_instance_poll(self.h, _ptr(buf), len(buf), C.byref(m)), "bd_instance_poll")
        return [int(v) for v in buf[:m.value]]

    def harvest(self, slot):
        # harvest copies and frees in one call, so size the buffer first
        cap = max(int(self.instance_counts()[slot]), 1)
        pos = np.empty((cap, 4), np.float32)
        sp = np.empty(cap, np.int32)
        n = C.c_size_t()
        L.check(self.lib.bd_instance_harvest(self.h, slot, _ptr(pos), _ptr(sp), cap, C.byref(n)), "harvest")
        m = min(n.value, cap)
        return np.ascontiguousarray(pos[:m, :3]), sp[:m]

    def cancel(self, slot):
        """Drop an admitted instance, frozen or running (bd_instance_cancel)."""
        L.check(self.lib.bd_instance_cancel(self.h, slot), "bd_instance_cancel")

    def instance_state(self, slot):
        s, f = C.c_uint32(), C.c_uint32()
        L.check(self.lib.bd_instance_state(self.h, slot, C.byref(s), C.byref(f)), "bd_instance_state")
        return s.value, f.value

    def set_launch_shape(self, block_stream=256, ctas_stream=4, block_pairs=256, ctas_pairs=4):
        L.check(self.lib.bd_set_launch_shape(self.h, block_stream, ctas_stream, block_pairs, ctas_pairs),
                "bd_set_launch_shape")

    def time_steps(self, n) -> float:
        """Device time in ms of n steps (CUDA events on the handle's stream)."""
        ms = C.c_float()
        L.check(self.lib.bd_time_steps(self.h, int(n), C.byref(ms)), "bd_time_steps", ok=(L.BD_OK, L.BD_ERR_EMPTY))
        return ms.value

    def profile_steps(self, n):
        """Summed device time per kernel over n steps: {kernel name: ms}."""
        buf = np.zeros(32, np.float32)
        k = C.c_int()
        L.check(self.lib.bd_profile_steps(self.h, int(n), _ptr(buf), 32, C.byref(k)), "bd_profile_steps")
        return {self.lib.bd_stage_name(self.h, i).decode(): float(buf[i]) for i in range(k.value)}

    def kernels_per_step(self) -> int:
        k = C.c_int()
        L.check(self.lib.bd_get_kernels_per_step(self.h, C.byref(k)), "kernels_per_step")
        return k.value

    def save_checkpoint(self, path):
        """The whole dynamic state, to resume bit for bit (bd_save_checkpoint)."""
        L.check(self.lib.bd_save_checkpoint(self.h, str(path).encode()), "bd_save_checkpoint")

    def load_checkpoint(self, path):
        """Resume from save_checkpoint's file on a handle built the same way."""
        L.check(self.lib.bd_load_checkpoint(self.h, str(path).encode()), "bd_load_checkpoint")

    def write_snapshot(self, path, binary=False):
        """Write the molecules to `path` (bd_write_snapshot)."""
        L.check(self.lib.bd_write_snapshot(self.h, str(path).encode(), 1 if binary else 0), "write_snapshot")

    def state_pointer(self):
        p = C.c_void_p()
        n = C.c_uint64()
        L.check(self.lib.bd_get_state_pointer(self.h, C.byref(p), C.byref(n)), "state_pointer")
        return p.value, n.value

    def close(self):
        if self.h:
            self.lib.bd_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def gauss_table(n=4096) -> np.ndarray:
    lib = L.load()
    out = np.zeros(n, np.float32)
    lib.bd_gauss_table(_ptr(out), n)
    return out


def numrxnrate(step, a, b):
    return L.load().bd_numrxnrate(step, a, b)


def actrxnrate(step, a):
    return L.load().bd_actrxnrate(step, a)


def bindingradius(rate, dt, difc, b, rel=0):
    return L.load().bd_bindingradius(rate, dt, difc, b, rel)


def unbindingradius(pgem, dt, difc, a):
    return L.load().bd_unbindingradius(pgem, dt, difc, a)
