"""ctypes binding of the C ABI in include/cellflow.h.

The library is the in-tree ``libcellflow.so`` built for sm_103a
(``libcellflow_bounds.so``, the bounds-checked build, when the environment
sets CELLFLOW_LIBRARY=bounds).  Loading fails loudly when it is missing:
there is no CPU fallback for the step.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / ("libcellflow_bounds.so" if os.environ.get("CELLFLOW_LIBRARY") == "bounds" else "libcellflow.so")

CF_OK = 0
CF_ERR_INVALID = -1
CF_ERR_CUDA = -2
CF_ERR_ALLOC = -3
CF_ERR_DOMAIN = -4
CF_ERR_DEVICE = -5
CF_ERR_CAPACITY = -6
CF_MAX_TYPES = 32
CF_MAX_PROX_CONN = 16
# Order of the parameter gradients of cf_rollout_backward (CF_GRAD_*).
GRAD_PARAMS = ("repulsion", "attraction", "k", "force_multiplier", "balance", "friction")

_ERR_NAMES = {
    CF_ERR_INVALID: "CF_ERR_INVALID",
    CF_ERR_CUDA: "CF_ERR_CUDA",
    CF_ERR_ALLOC: "CF_ERR_ALLOC",
    CF_ERR_DOMAIN: "CF_ERR_DOMAIN",
    CF_ERR_DEVICE: "CF_ERR_DEVICE",
    CF_ERR_CAPACITY: "CF_ERR_CAPACITY",
}


class CellFlowError(RuntimeError):
    """A CF_ERR_* status returned by the library."""

    def __init__(self, code: int, message: str, call: str):
        self.code = code
        super().__init__(f"{call}: {_ERR_NAMES.get(code, code)}: {message}")


class Particle(C.Structure):
    """cf_particle: the reference's 44-byte Particle (SimulationParams.h:6-12)."""

    _fields_ = [
        ("pos", C.c_float * 3),
        ("vel", C.c_float * 3),
        ("acc", C.c_float * 3),
        ("ptype", C.c_uint32),
        ("pad", C.c_float),
    ]


class Color(C.Structure):
    _fields_ = [("r", C.c_float), ("g", C.c_float), ("b", C.c_float)]


class StepParams(C.Structure):
    """cf_step_params: the physics fields of SimulationParams (SimulationParams.h:15-29)."""

    _fields_ = [
        ("radius", C.c_float),
        ("delta_t", C.c_float),
        ("friction", C.c_float),
        ("repulsion", C.c_float),
        ("attraction", C.c_float),
        ("k", C.c_float),
        ("balance", C.c_float),
        ("canvas_width", C.c_float),
        ("canvas_height", C.c_float),
        ("canvas_depth", C.c_float),
        ("num_particle_types", C.c_int),
        ("ratio_with_lfo", C.c_float),
        ("force_multiplier", C.c_float),
        ("max_expected_neighbors", C.c_int),
    ]


class GridInfo(C.Structure):
    _fields_ = [
        ("cells", C.c_int * 3),
        ("inv_cell", C.c_float * 3),
        ("r_max", C.c_float),
        ("generic_wrap", C.c_int),
        ("key_bits", C.c_int),
    ]


class DeviceView(C.Structure):
    _fields_ = [
        ("pos4", C.c_void_p),
        ("vel4", C.c_void_p),
        ("acc4", C.c_void_p),
        ("counts", C.c_void_p),
        ("n", C.c_int),
    ]


class PhaseTimes(C.Structure):
    _fields_ = [
        ("cell_list_ms", C.c_double),
        ("force_ms", C.c_double),
        ("steps", C.c_longlong),
        ("launches", C.c_longlong),
        ("adjoint_ms", C.c_double),
        ("adjoint_steps", C.c_longlong),
    ]


class Preset(C.Structure):
    """cf_preset: a parsed preset file (CellFlowWidget.cpp:1070-1259)."""

    _fields_ = [
        ("present", C.c_uint),
        ("particle_count", C.c_int),
        ("params", StepParams),
        ("force_range", C.c_float),
        ("force_bias", C.c_float),
        ("force_offset", C.c_float),
        ("ratio", C.c_float),
        ("lfo_a", C.c_float),
        ("lfo_s", C.c_float),
        ("spawn_region", C.c_float),
        ("n_radio", C.c_int),
        ("radio", C.c_float * CF_MAX_TYPES),
        ("n_raw", C.c_int),
        ("raw", C.c_float * (CF_MAX_TYPES * CF_MAX_TYPES)),
        ("n_colors", C.c_int),
        ("colors", Color * CF_MAX_TYPES),
        ("extra", C.c_char * 8192),
    ]


PRESET_BITS = {
    "PARTICLE_COUNT": 1 << 0, "numParticleTypes": 1 << 1, "radius": 1 << 2, "delta_t": 1 << 3,
    "friction": 1 << 4, "repulsion": 1 << 5, "attraction": 1 << 6, "k": 1 << 7, "balance": 1 << 8,
    "forceMultiplier": 1 << 9, "canvas": 1 << 10, "forceTransform": 1 << 11, "lfo": 1 << 12,
    "spawnRegionSize": 1 << 13, "radioByType": 1 << 14, "rawForceTable": 1 << 15, "particleColors": 1 << 16,
}

_W = C.c_void_p
_P = C.POINTER
_SIGNATURES = {
    "cf_last_error": (C.c_char_p, []),
    "cf_version": (C.c_char_p, []),
    "cf_kernel_launches": (C.c_longlong, []),
    "cf_set_device_memory_limit": (C.c_int, [C.c_size_t]),
    "cf_device_memory_in_use": (C.c_int, [_P(C.c_size_t)]),
    "cf_inject_cuda_error": (C.c_int, [C.c_char_p, C.c_int, C.c_int]),
    "cf_injection_pending": (C.c_int, []),
    "cf_default_params": (None, [_P(StepParams)]),
    "cf_create": (C.c_int, [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_uint64, _P(_W)]),
    "cf_destroy": (C.c_int, [_W]),
    "cf_set_stream": (C.c_int, [_W, C.c_void_p]),
    "cf_sync": (C.c_int, [_W]),
    "cf_particle_count": (C.c_int, [_W, _P(C.c_int)]),
    "cf_num_particle_types": (C.c_int, [_W, _P(C.c_int)]),
    "cf_set_particle_count": (C.c_int, [_W, C.c_int, C.c_uint64]),
    "cf_set_num_particle_types": (C.c_int, [_W, C.c_int, C.c_uint64]),
    "cf_initialize_particles": (C.c_int, [_W, C.c_uint64, C.c_float]),
    "cf_set_canvas": (C.c_int, [_W, C.c_float, C.c_float, C.c_float]),
    "cf_move_universe": (C.c_int, [_W, C.c_float, C.c_float, C.c_float]),
    "cf_get_particles": (C.c_int, [_W, C.c_void_p, C.c_int]),
    "cf_set_particles": (C.c_int, [_W, C.c_void_p, C.c_int]),
    "cf_get_state": (C.c_int, [_W, C.c_void_p, C.c_void_p, C.c_void_p]),
    "cf_set_state": (C.c_int, [_W, C.c_void_p, C.c_void_p, C.c_void_p]),
    "cf_get_neighbor_counts": (C.c_int, [_W, C.c_void_p, C.c_int]),
    "cf_device_buffers": (C.c_int, [_W, _P(DeviceView)]),
    "cf_get_raw_force_table": (C.c_int, [_W, C.c_void_p, C.c_int]),
    "cf_set_raw_force_table": (C.c_int, [_W, C.c_void_p, C.c_int]),
    "cf_regenerate_force_table": (C.c_int, [_W, C.c_uint64]),
    "cf_update_force_table": (C.c_int, [_W, C.c_float, C.c_float, C.c_float]),
    "cf_set_force_table": (C.c_int, [_W, C.c_void_p, C.c_int]),
    "cf_get_force_table": (C.c_int, [_W, C.c_void_p, C.c_int]),
    "cf_get_radio_by_type": (C.c_int, [_W, C.c_void_p, C.c_int]),
    "cf_set_radio_by_type": (C.c_int, [_W, C.c_void_p, C.c_int]),
    "cf_set_radio_by_type_value": (C.c_int, [_W, C.c_int, C.c_float]),
    "cf_rotate_radio_by_type": (C.c_int, [_W]),
    "cf_lfo_ratio": (C.c_float, [C.c_float, C.c_float, C.c_float, C.c_float]),
    "cf_step": (C.c_int, [_W, _P(StepParams), C.c_int]),
    "cf_step_host": (C.c_int, [_W, _P(StepParams), C.c_void_p, C.c_void_p, C.c_int]),
    "cf_get_grid": (C.c_int, [_W, _P(StepParams), _P(GridInfo)]),
    "cf_autotune_step": (C.c_int, [_W, _P(StepParams), C.c_int, _P(C.c_int)]),
    "cf_set_force_variant": (C.c_int, [_W, C.c_int]),
    "cf_debug_cell_list": (
        C.c_int,
        [_W, _P(StepParams), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int],
    ),
    "cf_work_counters": (C.c_int, [_W, _P(StepParams), _P(C.c_uint64), _P(C.c_uint64)]),
    "cf_force_work": (C.c_int, [_W, _P(StepParams), _P(C.c_uint64), _P(C.c_uint64)]),
    "cf_debug_bounds": (C.c_int, [_P(C.c_int), _P(C.c_int), C.c_char_p, C.c_int, _P(C.c_longlong),
                                  _P(C.c_longlong)]),
    "cf_debug_force_bad_item": (C.c_int, [_W, _P(StepParams), C.c_int]),
    "cf_proximity_edges": (C.c_int, [_W, C.c_float, C.c_int, C.c_void_p, C.c_int, _P(C.c_int)]),
    "cf_proximity_vertices_device": (
        C.c_int,
        [_W, C.c_float, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, _P(C.c_int)],
    ),
    "cf_triangle_mesh": (C.c_int, [_W, C.c_float, C.c_int, C.c_void_p, C.c_int, _P(C.c_int)]),
    "cf_triangle_mesh_device": (
        C.c_int,
        [_W, C.c_float, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, _P(C.c_int)],
    ),
    "cf_proximity_edges_noalloc": (
        C.c_int,
        [C.c_void_p, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_void_p, C.c_int,
         _P(C.c_int), C.c_void_p],
    ),
    "cf_batch_create": (C.c_int, [C.c_int, C.c_void_p, C.c_int, C.c_float, C.c_float, C.c_float, C.c_uint64,
                                  _P(_W)]),
    "cf_batch_destroy": (C.c_int, [_W]),
    "cf_batch_info": (C.c_int, [_W, _P(C.c_int), _P(C.c_int), C.c_void_p]),
    "cf_batch_world": (C.c_int, [_W, _P(_W)]),
    "cf_batch_set_state": (C.c_int, [_W, C.c_void_p, C.c_void_p, C.c_void_p]),
    "cf_batch_get_state": (C.c_int, [_W, C.c_void_p, C.c_void_p, C.c_void_p]),
    "cf_batch_set_force_tables": (C.c_int, [_W, C.c_void_p, C.c_int]),
    "cf_batch_step": (C.c_int, [_W, _P(StepParams), C.c_int]),
    "cf_batch_capture": (C.c_int, [_W, _P(StepParams), C.c_int]),
    "cf_batch_replay": (C.c_int, [_W]),
    "cf_batch_graph_info": (C.c_int, [_W, _P(C.c_int), _P(C.c_longlong)]),
    "cf_batch_autotune": (C.c_int, [_W, _P(StepParams), C.c_int, _P(C.c_int)]),
    "cf_batch_sync": (C.c_int, [_W]),
    "cf_batch_set_stream": (C.c_int, [_W, C.c_void_p]),
    "cf_rollout_forward": (C.c_int, [_W, _P(StepParams), C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                     C.c_void_p]),
    "cf_rollout_backward": (C.c_int, [_W, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                      C.c_void_p]),
    "cf_rdf": (C.c_int, [_W, C.c_void_p, C.c_int, C.c_float, C.c_void_p]),
    "cf_rdf_backward": (C.c_int, [_W, C.c_void_p, C.c_int, C.c_float, C.c_void_p, C.c_void_p]),
    "cf_preset_parse": (C.c_int, [C.c_char_p, C.c_size_t, _P(Preset)]),
    "cf_preset_apply": (C.c_int, [_W, _P(Preset), C.c_uint64, _P(StepParams)]),
    "cf_preset_write": (C.c_int, [_W, _P(Preset), C.c_char_p, C.c_size_t, _P(C.c_size_t)]),
    "cf_profile_enable": (C.c_int, [_W, C.c_int]),
    "cf_profile_read": (C.c_int, [_W, _P(PhaseTimes)]),
    "cf_measure_fp32_peak": (C.c_int, [_P(C.c_double)]),
}

_lib: C.CDLL | None = None


def load() -> C.CDLL:
    """Load libcellflow.so (raises if it is missing or incomplete)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`. "
            "There is no CPU fallback for the CellFlow step."
        )
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, call: str) -> None:
    if rc != CF_OK:
        msg = load().cf_last_error().decode(errors="replace")
        raise CellFlowError(rc, msg, call)


def declared_symbols() -> list[str]:
    """Names of the entry points this binding declares."""
    return sorted(_SIGNATURES)
