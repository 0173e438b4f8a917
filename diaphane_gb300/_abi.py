"""ctypes mirror of include/diaphane_gb300.h and the library loader.

The loader never falls back to anything: if the CUDA library has not been
built, importing the simulation API raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIBRARY = Path(__file__).resolve().parent / "libdiaphane_gb300.so"

DP_OK = 0
STATUS_NAMES = {0: "DP_OK", 1: "DP_ERR_INVALID", 2: "DP_ERR_LOSSY", 3: "DP_ERR_CUDA", 4: "DP_ERR_TIMEOUT",
                5: "DP_ERR_OOM", 6: "DP_ERR_UNSUPPORTED", 7: "DP_ERR_RANGE", 8: "DP_ERR_BUSY",
                9: "DP_ERR_NONFINITE"}
DP_ERR_INVALID, DP_ERR_LOSSY, DP_ERR_CUDA, DP_ERR_TIMEOUT = 1, 2, 3, 4
DP_ERR_OOM, DP_ERR_UNSUPPORTED, DP_ERR_RANGE, DP_ERR_BUSY = 5, 6, 7, 8
DP_ERR_NONFINITE = 9

DP_BOUNDARY_PEC, DP_BOUNDARY_ABSORBING = 0, 1
DP_SHAPE_BLOCK, DP_SHAPE_SPHERE, DP_SHAPE_SLAB = 0, 1, 2
DP_WAVE_RICKER, DP_WAVE_GAUSSIAN_PULSE, DP_WAVE_CONTINUOUS = 0, 1, 2
DP_SOURCE_POINT, DP_SOURCE_SHEET, DP_SOURCE_PLANE_WAVE, DP_SOURCE_PLANE_WAVE_BOX = 0, 1, 2, 3
DP_TABLE_MAGNETIC_GAINS, DP_TABLE_ELECTRIC_GAINS, DP_TABLE_CELL_CENTERS, DP_TABLE_ABSORBER = 0, 1, 2, 3
DP_TABLE_COEFFICIENTS, DP_TABLE_MATERIAL_INDEX, DP_TABLE_PRIMARY, DP_TABLE_DUAL = 4, 5, 6, 7
DP_MAP_TO_CELL, DP_MAP_TO_POSITION, DP_MAP_CELL_CONTAINING, DP_MAP_CELL_CENTER = 0, 1, 2, 3
DP_KERNEL_AUTO, DP_KERNEL_FUSED, DP_KERNEL_NAIVE = 0, 1, 2
DP_FIELD_ELECTRIC, DP_FIELD_MAGNETIC, DP_FIELD_INTENSITY = 0, 1, 2

F3 = C.c_float * 3
U3 = C.c_uint32 * 3


class dp_refinement(C.Structure):
    _fields_ = [("center", F3), ("size", F3), ("cell_size", C.c_float)]


class dp_grid_spec(C.Structure):
    _fields_ = [("extent", U3), ("cell_size", C.c_float), ("courant", C.c_float), ("max_ratio", C.c_float),
                ("refinement_count", C.c_uint32), ("refinements", C.POINTER(dp_refinement))]


class dp_boundary(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("thickness", C.c_uint32), ("target_reflection", C.c_float)]


class dp_material(C.Structure):
    _fields_ = [("relative_permittivity", C.c_float), ("relative_permeability", C.c_float),
                ("conductivity", C.c_float), ("magnetic_loss", C.c_float)]


class dp_shape(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("material", C.c_uint32), ("center", F3), ("size", F3),
                ("radius", C.c_float), ("axis", C.c_uint32), ("offset", C.c_float), ("thickness", C.c_float)]


class dp_waveform(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("frequency", C.c_float), ("duration_cycles", C.c_float),
                ("ramp_cycles", C.c_float), ("delay", C.c_float)]


class dp_source(C.Structure):
    _fields_ = [("shape", C.c_uint32), ("polarization", C.c_uint32), ("at", F3), ("velocity", F3),
                ("axis", C.c_uint32), ("offset", C.c_float), ("waist", C.c_float), ("amplitude", C.c_float),
                ("waveform", dp_waveform), ("box_low", F3), ("box_high", F3)]


class dp_scene_desc(C.Structure):
    _fields_ = [("grid", dp_grid_spec), ("boundary", dp_boundary),
                ("material_count", C.c_uint32), ("materials", C.POINTER(dp_material)),
                ("shape_count", C.c_uint32), ("shapes", C.POINTER(dp_shape)),
                ("source_count", C.c_uint32), ("sources", C.POINTER(dp_source))]


class dp_grid_info(C.Structure):
    _fields_ = [("extent", U3), ("size", F3), ("time_step", C.c_float), ("finest", C.c_float),
                ("coarsest", C.c_float), ("worst_ratio", C.c_float), ("reference_cell_size", C.c_float)]


class dp_scene_info(C.Structure):
    _fields_ = [("extent", U3), ("material_count", C.c_uint32), ("time_step", C.c_float),
                ("courant", C.c_float), ("absorber_peak", C.c_float), ("reversible", C.c_int32),
                ("index_bytes", C.c_uint32)]


class dp_injection(C.Structure):
    _fields_ = [("origin", U3), ("extent", U3), ("component", C.c_uint32), ("magnetic", C.c_uint32),
                ("value", C.c_float), ("inverse_waist_squared", C.c_float), ("center", F3)]


class dp_batch_options(C.Structure):
    _fields_ = [("device", C.c_int32), ("chunk_steps", C.c_uint32), ("arena_bytes", C.c_uint64),
                ("max_scenes", C.c_uint32), ("use_graphs", C.c_uint32), ("cells_per_lane", C.c_uint32),
                ("unit_planes", C.c_uint32), ("skip_finite_check", C.c_uint32), ("axis_order", C.c_uint32)]


class dp_options(C.Structure):
    _fields_ = [("device", C.c_int32), ("kernel", C.c_uint32), ("tile_y", C.c_uint32), ("z_chunk", C.c_uint32),
                ("cells_per_lane", C.c_uint32), ("ring_slots", C.c_uint32)]


# Every entry point declared in include/diaphane_gb300.h: (name, restype, argtypes).
_P = C.c_void_p
class dp_view(C.Structure):
    _fields_ = [("yaw", C.c_float), ("pitch", C.c_float), ("distance", C.c_float), ("fov", C.c_float),
                ("mode", C.c_uint32), ("gain", C.c_float), ("log_strength", C.c_float), ("scrub", C.c_int32),
                ("played", C.c_float), ("window_start", C.c_float)]


DP_VIEW_ENERGY, DP_VIEW_ELECTRIC, DP_VIEW_MAGNETIC, DP_VIEW_MAGNITUDE = 0, 1, 2, 3
DP_VIEW_FIELDS, DP_VIEW_GRID, DP_VIEW_RIBBONS, DP_VIEW_INTENSITY = 4, 5, 6, 7


class dp_tuning(C.Structure):
    _fields_ = [("cells_per_lane", C.c_uint32), ("tile_y", C.c_uint32), ("ring_slots", C.c_uint32),
                ("z_chunk", C.c_uint32), ("ms_per_step", C.c_float), ("candidates", C.c_uint32)]


class dp_seek(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("replayed", C.c_uint64), ("at", C.c_uint64)]


DP_SEEK_UNCHANGED, DP_SEEK_FORWARD, DP_SEEK_KEYFRAME, DP_SEEK_START = 0, 1, 2, 3

SIGNATURES = [
    ("dp_last_error", C.c_char_p, []),
    ("dp_status_string", C.c_char_p, [C.c_int]),
    ("dp_grid_resolve", C.c_int, [C.POINTER(dp_grid_spec), C.POINTER(dp_grid_info)]),
    ("dp_grid_map", C.c_int, [C.POINTER(dp_grid_spec), C.c_uint32, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    ("dp_scene_create", C.c_int, [C.POINTER(dp_scene_desc), C.POINTER(_P)]),
    ("dp_scene_destroy", None, [_P]),
    ("dp_scene_info_get", C.c_int, [_P, C.POINTER(dp_scene_info)]),
    ("dp_scene_table", C.c_int, [_P, C.c_uint32, _P, C.c_size_t]),
    ("dp_scene_injections", C.c_int, [_P, C.c_float, C.POINTER(dp_injection), C.c_uint32, C.POINTER(C.c_uint32)]),
    ("dp_sim_create", C.c_int, [_P, C.POINTER(dp_options), C.POINTER(_P)]),
    ("dp_sim_destroy", None, [_P]),
    ("dp_sim_advance", C.c_int, [_P, C.c_uint64]),
    ("dp_sim_reverse", C.c_int, [_P, C.c_uint64]),
    ("dp_sim_reset", C.c_int, [_P]),
    ("dp_sim_wait", C.c_int, [_P, C.c_uint32]),
    ("dp_sim_step_count", C.c_uint64, [_P]),
    ("dp_sim_time", C.c_float, [_P]),
    ("dp_sim_read_field", C.c_int, [_P, C.c_uint32, _P, C.c_size_t]),
    ("dp_sim_write_field", C.c_int, [_P, C.c_uint32, _P, C.c_size_t]),
    ("dp_sim_restore", C.c_int, [_P, C.c_uint64, _P, _P, C.c_size_t]),
    ("dp_sim_set_accumulate_intensity", C.c_int, [_P, C.c_int]),
    ("dp_sim_accumulated_steps", C.c_uint64, [_P]),
    ("dp_sim_device_ptr", C.c_int, [_P, C.c_uint32, C.POINTER(_P)]),
    ("dp_sim_stream", C.c_int, [_P, C.POINTER(_P)]),
    ("dp_sim_bytes_per_step", C.c_uint64, [_P]),
    ("dp_sim_field_bytes", C.c_uint64, [_P]),
    ("dp_sim_energy", C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("dp_sim_is_finite", C.c_int, [_P, C.POINTER(C.c_int32)]),
    ("dp_sim_is_reversible", C.c_int32, [_P]),
    ("dp_batch_create", C.c_int, [C.POINTER(dp_batch_options), C.POINTER(_P)]),
    ("dp_batch_destroy", None, [_P]),
    ("dp_batch_add", C.c_int, [_P, _P, C.c_uint64, C.c_int32, C.POINTER(C.c_uint32), C.c_uint32,
                               C.POINTER(C.c_uint64)]),
    ("dp_batch_remove", C.c_int, [_P, C.c_uint64]),
    ("dp_batch_advance_chunk", C.c_int, [_P, C.POINTER(C.c_uint32)]),
    ("dp_batch_wait", C.c_int, [_P, C.c_uint32]),
    ("dp_batch_status", C.c_int, [_P, C.c_uint64, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    ("dp_batch_fault", C.c_int, [_P, C.c_uint64, C.POINTER(C.c_int), C.POINTER(C.c_uint64)]),
    ("dp_batch_read_field", C.c_int, [_P, C.c_uint64, C.c_uint32, _P, C.c_size_t]),
    ("dp_batch_read_probes", C.c_int, [_P, C.c_uint64, _P, C.c_size_t]),
    ("dp_batch_memory", C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    ("dp_scene_batch_bytes", C.c_uint64, [_P, C.c_uint32, C.c_uint64]),
    ("dp_batch_launch_count", C.c_uint64, [_P]),
    ("dp_batch_layout", C.c_int, [_P, C.c_uint64, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    ("dp_energy_noalloc", C.c_int, [_P, _P, C.c_uint32, _P, C.c_uint32, C.c_uint32, _P, C.c_uint32, _P, _P,
                                     C.POINTER(C.c_uint32), _P, _P]),
    ("dp_sim_kernel", C.c_uint32, [_P]),
    ("dp_sim_row_pitch", C.c_uint32, [_P]),
    ("dp_sim_launch_count", C.c_uint64, [_P]),
    ("dp_scene_raster", C.c_int, [_P, _P, C.c_uint32, _P]),
    ("dp_scene_cell_lookup", C.c_int, [_P, C.c_uint32, _P, C.c_size_t]),
    ("dp_scene_lookup_samples", C.c_uint32, [_P]),
    ("dp_sim_energy_density", C.c_int, [_P, _P, C.c_size_t]),
    ("dp_sim_sample", C.c_int, [_P, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_float)]),
    ("dp_sim_autotune", C.c_int, [_P, C.c_uint32, C.POINTER(dp_tuning)]),
    ("dp_sim_plan", C.c_int, [_P, C.POINTER(dp_tuning)]),
    ("dp_tune_cache_export", C.c_int, [C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    ("dp_tune_cache_import", C.c_int, [C.c_char_p]),
    ("dp_tune_cache_clear", None, []),
    ("dp_sim_set_probes", C.c_int, [_P, _P, C.c_uint32, C.c_uint64]),
    ("dp_sim_read_probes", C.c_int, [_P, C.c_uint64, C.c_uint64, _P, C.c_size_t]),
    ("dp_sim_read_field_async", C.c_int, [_P, C.c_uint32, _P, C.c_size_t]),
    ("dp_keyframes_create", C.c_int, [_P, C.c_uint64, C.c_uint32, C.POINTER(_P)]),
    ("dp_keyframes_destroy", None, [_P]),
    ("dp_keyframes_observe", C.c_int, [_P]),
    ("dp_keyframes_seek", C.c_int, [_P, C.c_uint64, C.POINTER(dp_seek)]),
    ("dp_keyframes_clear", C.c_int, [_P]),
    ("dp_keyframes_count", C.c_uint32, [_P]),
    ("dp_keyframes_earliest", C.c_int, [_P, C.POINTER(C.c_uint64)]),
    ("dp_keyframes_bytes", C.c_uint64, [_P]),
    ("dp_view_default", dp_view, []),
    ("dp_renderer_create", C.c_int, [_P, C.c_uint32, C.c_uint32, C.POINTER(_P)]),
    ("dp_renderer_destroy", None, [_P]),
    ("dp_renderer_measure", C.c_int, [_P]),
    ("dp_renderer_draw", C.c_int, [_P, C.POINTER(dp_view), C.c_int32]),
    ("dp_renderer_pixels", C.c_int, [_P, _P, C.c_size_t]),
    ("dp_renderer_image", C.c_int, [_P, C.POINTER(_P)]),
    ("dp_renderer_state", C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_uint32)]),
    ("dp_sim64_create", C.c_int, [_P, C.c_int32, C.POINTER(_P)]),
    ("dp_sim64_destroy", None, [_P]),
    ("dp_sim64_advance", C.c_int, [_P, C.c_uint64]),
    ("dp_sim64_wait", C.c_int, [_P, C.c_uint32]),
    ("dp_sim64_step_count", C.c_uint64, [_P]),
    ("dp_sim64_read_field", C.c_int, [_P, C.c_uint32, _P, C.c_size_t]),
    ("dp_sim64_energy", C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
]


class DiaphaneError(RuntimeError):
    """A non-OK dp_status, carrying the library's message."""

    def __init__(self, status: int, message: str):
        self.status = status
        self.name = STATUS_NAMES.get(status, str(status))
        super().__init__(f"{self.name}: {message}")


_lib = None


def lib() -> C.CDLL:
    """The loaded CUDA library.  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIBRARY.exists():
            raise ImportError(
                f"{LIBRARY} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`. "
                "There is no CPU fallback.")
        handle = C.CDLL(str(LIBRARY))
        for name, restype, argtypes in SIGNATURES:
            fn = getattr(handle, name)
            fn.restype = restype
            fn.argtypes = argtypes
        _lib = handle
    return _lib


def check(status: int) -> None:
    if status != DP_OK:
        message = lib().dp_last_error().decode(errors="replace")
        raise DiaphaneError(status, message)
