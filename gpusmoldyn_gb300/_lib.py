"""ctypes binding of include/gpusmoldyn.h (libgpusmoldyn.so, built in-tree).

The library is the product: there is no Python or CPU fallback.  Loading
fails loudly when the shared object is missing.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgpusmoldyn.so")

# status codes (include/gpusmoldyn.h)
BD_OK = 0
BD_ERR_NEGATIVE_RATE = 1
BD_ERR_STATE_DEPENDENT = 2
BD_ERR_ZERO_DIFFUSION = 4
BD_ERR_ILLEGAL_UNBIND = 7
BD_ERR_PGEM_UNATTAINABLE = 8
BD_ERR_INVALID_ARGUMENT = 16
BD_ERR_NOT_FINALIZED = 17
BD_ERR_ALREADY_FINALIZED = 18
BD_ERR_CAPACITY = 19
BD_ERR_EMPTY = 20
BD_ERR_CUDA = 21
BD_ERR_TIMEOUT = 22
BD_ERR_NO_DEVICE = 23
BD_ERR_DEVICE_STATE = 24
BD_ERR_UNSUPPORTED = 25

BD_DEVICE_NONE = -1

BD_NORMALS_BOXMULLER = 0
BD_NORMALS_TABLE = 1

BD_PAIR_LAST = 0
BD_PAIR_CHANNELS = 1

BD_SORT_AUTO = 0
BD_SORT_COMPACT = 1
BD_SORT_BINNED = 2

BD_PP_DEFAULT = 0
BD_PP_PGEM = 1
BD_PP_PGEMMAX = 2
BD_PP_UNBINDRAD = 3
BD_PP_OFFSET0 = 4

BD_PANEL_RECT = 0
BD_PANEL_TRI = 1
BD_PANEL_SPH = 2
BD_PANEL_CYL = 3
BD_PANEL_HEMI = 4
BD_PANEL_DISK = 5

BD_FACE_FRONT = 0
BD_FACE_BACK = 1
BD_FACE_BOTH = 2

BD_SURF_TRANSMIT = 0
BD_SURF_REFLECT = 1
BD_SURF_ABSORB = 2

BD_ALL_SPECIES = -1

DEAD = 0xFFFFFFFF


class bd_config(C.Structure):
    _fields_ = [("box_lo", C.c_float * 3), ("box_hi", C.c_float * 3), ("dt", C.c_float),
                ("seed", C.c_uint64), ("capacity", C.c_uint64), ("cell_size", C.c_float),
                ("cell_occupancy", C.c_float), ("normal_mode", C.c_int), ("device", C.c_int),
                ("pair_capacity", C.c_uint32), ("sort_mode", C.c_uint32), ("pair_mode", C.c_uint32),
                ("reserved", C.c_uint32 * 5)]


class bd_reaction_info(C.Structure):
    _fields_ = [("order", C.c_int), ("nprod", C.c_int), ("reactants", C.c_int * 2), ("products", C.c_int * 2),
                ("rate", C.c_float), ("prob", C.c_float), ("bind_radius", C.c_float),
                ("unbind_radius", C.c_float), ("geminate_prob", C.c_float), ("product_offsets", C.c_float * 2),
                ("reverse", C.c_int), ("flags", C.c_int), ("channel_threshold", C.c_float)]


class bd_instance_desc(C.Structure):
    _fields_ = [("box_lo", C.c_float * 3), ("box_hi", C.c_float * 3), ("seed", C.c_uint64),
                ("d_scale", C.c_float), ("k2_scale", C.c_float), ("cell_size", C.c_float),
                ("reserved", C.c_uint32 * 3)]


class bd_model_info(C.Structure):
    _fields_ = [("time_start", C.c_double), ("time_stop", C.c_double), ("steps", C.c_uint64),
                ("n_molecules", C.c_uint64), ("n_species", C.c_int), ("n_reactions", C.c_int)]


class bd_panel(C.Structure):
    _fields_ = [("shape", C.c_int), ("axis", C.c_int), ("front", C.c_int), ("p", C.c_float * 10)]


class bd_panel_info(C.Structure):
    _fields_ = [("shape", C.c_int), ("surface", C.c_int), ("axis", C.c_int), ("front", C.c_float),
                ("a", C.c_float * 3), ("r", C.c_float), ("r2", C.c_float), ("n", C.c_float * 3),
                ("len", C.c_float), ("v1", C.c_float * 3), ("v2", C.c_float * 3), ("bounds", C.c_float * 4)]


H = C.c_void_p
P = C.c_void_p
_SIGS = {
    "bd_config_default": (None, [C.POINTER(bd_config)]),
    "bd_create": (C.c_int, [C.POINTER(bd_config), C.POINTER(H)]),
    "bd_create_ensemble": (C.c_int, [C.POINTER(bd_config), C.POINTER(bd_instance_desc), C.c_int, C.POINTER(H)]),
    "bd_destroy": (C.c_int, [H]),
    "bd_add_species": (C.c_int, [H, C.c_float, C.POINTER(C.c_int)]),
    "bd_add_reaction": (C.c_int, [H, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_float,
                                  C.POINTER(C.c_int)]),
    "bd_set_product_placement": (C.c_int, [H, C.c_int, C.c_int, C.c_float]),
    "bd_set_reaction_probability": (C.c_int, [H, C.c_int, C.c_float]),
    "bd_finalize": (C.c_int, [H]),
    "bd_get_reaction_info": (C.c_int, [H, C.c_int, C.POINTER(bd_reaction_info)]),
    "bd_get_instance_reaction_info": (C.c_int, [H, C.c_int, C.c_int, C.POINTER(bd_reaction_info)]),
    "bd_get_counts": (C.c_int, [H, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "bd_set_particles": (C.c_int, [H, P, P, C.c_size_t]),
    "bd_set_ensemble_particles": (C.c_int, [H, P, P, P, C.c_int]),
    "bd_get_count": (C.c_int, [H, C.POINTER(C.c_uint64)]),
    "bd_get_particles": (C.c_int, [H, P, P, C.c_size_t, C.POINTER(C.c_size_t)]),
    "bd_get_instance_particles": (C.c_int, [H, C.c_int, P, P, C.c_size_t, C.POINTER(C.c_size_t)]),
    "bd_instance_cancel": (C.c_int, [H, C.c_int]),
    "bd_get_instance_counts": (C.c_int, [H, P, C.c_int]),
    "bd_get_species_counts": (C.c_int, [H, C.c_int, P, C.c_int]),
    "bd_measure_msd": (C.c_int, [H, C.c_int, C.c_int, P, P, C.c_int]),
    "bd_get_state_pointer": (C.c_int, [H, C.POINTER(C.c_void_p), C.POINTER(C.c_uint64)]),
    "bd_step": (C.c_int, [H, C.c_int]),
    "bd_step_async": (C.c_int, [H, C.c_int, P]),
    "bd_synchronize": (C.c_int, [H]),
    "bd_get_step": (C.c_int, [H, C.POINTER(C.c_uint64)]),
    "bd_get_event_counts": (C.c_int, [H, P, C.c_int]),
    "bd_time_steps": (C.c_int, [H, C.c_int, C.POINTER(C.c_float)]),
    "bd_profile_steps": (C.c_int, [H, C.c_int, P, C.c_int, C.POINTER(C.c_int)]),
    "bd_stage_name": (C.c_char_p, [H, C.c_int]),
    "bd_get_kernels_per_step": (C.c_int, [H, C.POINTER(C.c_int)]),
    "bd_debug_get_slots": (C.c_int, [H, P, P, C.c_size_t, C.POINTER(C.c_size_t)]),
    "bd_debug_get_cells": (C.c_int, [H, P, C.c_size_t, C.POINTER(C.c_size_t)]),
    "bd_debug_withhold_scan": (C.c_int, [H, C.c_int]),
    "bd_debug_withhold_match": (C.c_int, [H, C.c_int]),
    "bd_debug_get_pairs": (C.c_int, [H, P, C.c_size_t, C.POINTER(C.c_size_t)]),
    "bd_get_grid": (C.c_int, [H, C.c_int, P, P, P]),
    "bd_get_poisson_cdf": (C.c_int, [H, C.c_int, C.c_int, P, C.c_size_t, C.POINTER(C.c_int),
                                     C.POINTER(C.c_size_t)]),
    "bd_get_species_d": (C.c_int, [H, C.c_int, C.c_int, C.POINTER(C.c_float)]),
    "bd_set_cell_size": (C.c_int, [H, C.c_float]),
    "bd_set_launch_shape": (C.c_int, [H, C.c_int, C.c_int, C.c_int, C.c_int]),
    "bd_create_server": (C.c_int, [C.POINTER(bd_config), C.c_int, C.POINTER(H)]),
    "bd_instance_admit": (C.c_int, [H, C.POINTER(bd_instance_desc), P, P, C.c_size_t, C.c_uint32,
                                    C.POINTER(C.c_int)]),
    "bd_instance_poll": (C.c_int, [H, P, C.c_int, C.POINTER(C.c_int)]),
    "bd_instance_harvest": (C.c_int, [H, C.c_int, P, P, C.c_size_t, C.POINTER(C.c_size_t)]),
    "bd_instance_state": (C.c_int, [H, C.c_int, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "bd_cell_sort_static": (C.c_int, [P, C.c_uint64, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                      C.POINTER(C.c_uint32), P, P, P]),
    "bd_get_config": (C.c_int, [H, C.POINTER(bd_config)]),
    "bd_save_checkpoint": (C.c_int, [H, C.c_char_p]),
    "bd_load_checkpoint": (C.c_int, [H, C.c_char_p]),
    "bd_add_surface": (C.c_int, [H, C.POINTER(C.c_int)]),
    "bd_set_surface_action": (C.c_int, [H, C.c_int, C.c_int, C.c_int, C.c_int]),
    "bd_get_surface_action": (C.c_int, [H, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "bd_add_panel": (C.c_int, [H, C.c_int, C.POINTER(bd_panel), C.POINTER(C.c_int)]),
    "bd_get_panel": (C.c_int, [H, C.c_int, C.POINTER(bd_panel_info)]),
    "bd_get_surface_counts": (C.c_int, [H, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "bd_write_snapshot": (C.c_int, [H, C.c_char_p, C.c_int]),
    "bd_set_species_name": (C.c_int, [H, C.c_int, C.c_char_p]),
    "bd_find_species": (C.c_int, [H, C.c_char_p, C.POINTER(C.c_int)]),
    "bd_set_reaction_name": (C.c_int, [H, C.c_int, C.c_char_p]),
    "bd_find_reaction": (C.c_int, [H, C.c_char_p, C.POINTER(C.c_int)]),
    "bd_create_from_model": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(H), C.POINTER(bd_model_info), C.c_char_p,
                                       C.c_size_t]),
    "bd_create_from_model_file": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(H), C.POINTER(bd_model_info),
                                            C.c_char_p, C.c_size_t]),
    "bd_numrxnrate": (C.c_double, [C.c_double, C.c_double, C.c_double]),
    "bd_actrxnrate": (C.c_double, [C.c_double, C.c_double]),
    "bd_bindingradius": (C.c_double, [C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]),
    "bd_unbindingradius": (C.c_double, [C.c_double, C.c_double, C.c_double, C.c_double]),
    "bd_gauss_table": (C.c_int, [P, C.c_int]),
    "bd_status_string": (C.c_char_p, [C.c_int]),
    "bd_version": (C.c_char_p, []),
}

_lib = None


def load(path: str | None = None):
    """Load libgpusmoldyn.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with gpusmoldyn_gb300.build.build()")
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return sorted(_SIGS)


class BDError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        lib = load()
        msg = lib.bd_status_string(code).decode()
        super().__init__(f"{what}: status {code} ({msg})" if what else f"status {code} ({msg})")
        self.code = code


def check(code: int, what: str = "", ok=(BD_OK,)):
    if code not in ok:
        raise BDError(code, what)
    return code
