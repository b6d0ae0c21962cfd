"""ctypes binding of libbbg.so (include/bbg.h).

The shared library is built in-tree by ``bubbles_gb300.build``; loading never falls
back to anything else -- a missing or unloadable library raises.
"""
import ctypes
import os

from . import build as _build

OK = 0
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of device memory",
          4: "capacity exceeded", 5: "invalid solver state", 6: "no CUDA device", 7: "not found"}

SOLVER_PCISPH, SOLVER_SPH = 0, 1
PCISPH_AS_SHIPPED, PCISPH_TOLERANCE = 0, 1
PRESSURE_INIT_ZERO, PRESSURE_INIT_PREVIOUS, PRESSURE_INIT_LEARNED = 0, 1, 2
WARM_CLAMP_TOTAL, WARM_MONOTONE = 0, 1
SHAPE_BOX, SHAPE_SPHERE, SHAPE_SDF = 1, 2, 3
MAX_COLLIDERS = 16

FIELD_POSITION, FIELD_VELOCITY, FIELD_FORCE, FIELD_INTERACTION = 0, 1, 2, 3
FIELD_DENSITY, FIELD_PRESSURE, FIELD_PRED_POSITION = 4, 5, 6
FIELD_PRESSURE_FORCE, FIELD_PRED_DENSITY, FIELD_DENSITY_ERROR = 8, 9, 10
FIELD_DIVERGENCE = 11
FRAME_POSITION, FRAME_VELOCITY, FRAME_DENSITY, FRAME_MASS = 0x01, 0x02, 0x04, 0x20
VECTOR_FIELDS = {FIELD_POSITION, FIELD_VELOCITY, FIELD_FORCE, FIELD_INTERACTION,
                 FIELD_PRED_POSITION, FIELD_PRESSURE_FORCE}


class SolverDesc(ctypes.Structure):
    _fields_ = [("solver_kind", ctypes.c_int),
                ("eos_exponent", ctypes.c_double),
                ("negative_pressure_scale", ctypes.c_double),
                ("viscosity", ctypes.c_double),
                ("pseudo_viscosity", ctypes.c_double),
                ("sound_speed", ctypes.c_double),
                ("drag_coefficient", ctypes.c_double),
                ("gravity", ctypes.c_double * 3),
                ("target_density", ctypes.c_double),
                ("target_spacing", ctypes.c_double),
                ("relative_kernel_radius", ctypes.c_double),
                ("mass", ctypes.c_double),
                ("domain_min", ctypes.c_double * 3),
                ("domain_max", ctypes.c_double * 3),
                ("grid_spacing_scale", ctypes.c_double),
                ("time_step_limit_scale", ctypes.c_double),
                ("pcisph_mode", ctypes.c_int),
                ("max_iterations", ctypes.c_int),
                ("max_density_error_ratio", ctypes.c_double),
                ("device", ctypes.c_int),
                ("pressure_init", ctypes.c_int),
                ("warm_rule", ctypes.c_int),
                ("warm_scale", ctypes.c_double)]


MLP_PARAMS = 4545


class MlpDesc(ctypes.Structure):
    _fields_ = [("train_substeps", ctypes.c_int),
                ("batch", ctypes.c_int),
                ("steps_per_substep", ctypes.c_int),
                ("learning_rate", ctypes.c_double),
                ("beta1", ctypes.c_double),
                ("beta2", ctypes.c_double),
                ("epsilon", ctypes.c_double),
                ("seed", ctypes.c_ulonglong),
                ("expectile", ctypes.c_double),
                ("finetune_steps", ctypes.c_int),
                ("refresh_interval", ctypes.c_int)]


class SceneDesc(ctypes.Structure):
    _fields_ = [("count", ctypes.c_int),
                ("box_min", ctypes.c_double * 3),
                ("box_max", ctypes.c_double * 3)]


class Tuning(ctypes.Structure):
    _fields_ = [("block_size", ctypes.c_int), ("batch_np", ctypes.c_int),
                ("batch_pd", ctypes.c_int), ("batch_pf", ctypes.c_int), ("prune", ctypes.c_int),
                ("particles_per_thread", ctypes.c_int), ("tile_order", ctypes.c_int),
                ("batch_worklist", ctypes.c_int)]


class Shape(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int), ("reverse", ctypes.c_int),
                ("center", ctypes.c_double * 3), ("size", ctypes.c_double * 3),
                ("friction", ctypes.c_double)]


class SdfGrid(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_int * 3), ("origin", ctypes.c_double * 3), ("spacing", ctypes.c_double * 3),
                ("bounded", ctypes.c_int), ("bounds_min", ctypes.c_double * 3),
                ("bounds_max", ctypes.c_double * 3)]


class EmitterDesc(ctypes.Structure):
    _fields_ = [("shape", Shape), ("use_bounds", ctypes.c_int),
                ("bounds_min", ctypes.c_double * 3), ("bounds_max", ctypes.c_double * 3),
                ("spacing", ctypes.c_double), ("jitter", ctypes.c_double),
                ("initial_velocity", ctypes.c_double * 3), ("max_particles", ctypes.c_int)]


class StepStats(ctypes.Structure):
    _fields_ = [("substeps", ctypes.c_int),
                ("iterations", ctypes.c_int),
                ("max_iterations_in_substep", ctypes.c_int),
                ("not_converged", ctypes.c_int),
                ("last_dt", ctypes.c_double),
                ("max_density_error_ratio", ctypes.c_double),
                ("mean_density_error_ratio", ctypes.c_double),
                ("neighbor_overflow", ctypes.c_int),
                ("out_of_grid", ctypes.c_int),
                ("max_force", ctypes.c_double),
                ("crowded", ctypes.c_int),
                ("nonfinite", ctypes.c_int)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class BbgError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s (%d): %s" % (STATUS.get(status, "?"), status, message))
        self.status = status


_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int
_FP = ctypes.POINTER(ctypes.c_float)
_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
_UP = ctypes.POINTER(ctypes.c_uint32)

# name -> argument types (every function returns int status unless listed in _RES)
SIGNATURES = {
    "bbg_device_count": [_IP],
    "bbg_solver_desc_default": [ctypes.POINTER(SolverDesc), _I],
    "bbg_build_grid": [_DP, _DP, _D, _D, _IP, _DP],
    "bbg_compute_mass": [_I, _D, _D, _D, _DP],
    "bbg_compute_delta_denom": [_D, _D, _DP],
    "bbg_create": [ctypes.POINTER(SolverDesc), _I, ctypes.POINTER(_P)],
    "bbg_destroy": [_P],
    "bbg_set_colliders": [_P, ctypes.POINTER(Shape), _I],
    "bbg_upload_particles": [_P, _FP, _FP, _I],
    "bbg_upload_particles_device": [_P, _P, _P, _I],
    "bbg_setup": [_P],
    "bbg_set_stream": [_P, _P],
    "bbg_synchronize": [_P],
    "bbg_advance": [_P, _D, ctypes.POINTER(StepStats)],
    "bbg_advance_time_step": [_P, _D, ctypes.POINTER(StepStats)],
    "bbg_get_stats": [_P, ctypes.POINTER(StepStats)],
    "bbg_update_grid_distribution": [_P],
    "bbg_compute_particle_interaction": [_P],
    "bbg_compute_density": [_P, _I],
    "bbg_compute_non_pressure_force": [_P],
    "bbg_compute_pressure_force": [_P, _D],
    "bbg_time_integration": [_P, _D],
    "bbg_compute_pseudo_viscosity_interpolation": [_P, _D],
    "bbg_compute_pressure_force_and_integrate": [_P, _D, _D, _D, _I, ctypes.POINTER(StepStats)],
    "bbg_compute_delta": [_P, _D, _DP],
    "bbg_predict_velocity_and_position": [_P, _D, _I],
    "bbg_predict_pressure": [_P, _D],
    "bbg_predict_pressure_force": [_P],
    "bbg_accumulate_and_integrate": [_P, _D],
    "bbg_compute_number_of_time_steps": [_P, _D, _D, ctypes.POINTER(ctypes.c_uint)],
    "bbg_particle_count": [_P, _IP],
    "bbg_get_field": [_P, _I, _FP],
    "bbg_set_field": [_P, _I, _FP],
    "bbg_download": [_P, _FP, _FP],
    "bbg_download_device": [_P, _P, _P],
    "bbg_get_scalars": [_P, _DP],
    "bbg_get_grid": [_P, _IP, _DP],
    "bbg_dump_grid": [_P, _UP, _UP, _UP],
    "bbg_neighbor_counts": [_P, _IP],
    "bbg_neighbor_lists": [_P, _I, _IP, _IP],
    "bbg_profiler_enable": [_P, _I],
    "bbg_use_cuda_graphs": [_P, _I],
    "bbg_grid_sort_noalloc": [_P, _I, _DP, _DP, _D, _D, _P, _P, _P, _P, _P],
    "bbg_get_tuning": [_P, ctypes.POINTER(Tuning)],
    "bbg_set_tuning": [_P, ctypes.POINTER(Tuning)],
    "bbg_batch_create": [ctypes.POINTER(SolverDesc), ctypes.POINTER(SceneDesc), _I, ctypes.POINTER(_P)],
    "bbg_batch_scene_count": [_P, _IP],
    "bbg_batch_layout": [_P, _DP],
    "bbg_batch_upload": [_P, _FP, _FP],
    "bbg_batch_download": [_P, _FP, _FP],
    "bbg_batch_scene_stats": [_P, _IP, _DP],
    "bbg_frame_text": [_P, _I, ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)],
    "bbg_frame_append": [_P, _I, ctypes.c_char_p],
    "bbg_format_g": [ctypes.c_float, ctypes.c_char_p, _IP],
    "bbg_frame_load": [_P, ctypes.c_char_p, _IP],
    "bbg_frame_load_text": [_P, ctypes.c_char_p, ctypes.c_size_t, _IP],
    "bbg_frame_find_section": [ctypes.c_char_p, ctypes.c_size_t, _IP, _IP, ctypes.POINTER(ctypes.c_size_t),
                               ctypes.POINTER(ctypes.c_size_t)],
    "bbg_emitter_desc_default": [ctypes.POINTER(EmitterDesc)],
    "bbg_emit_volume": [_P, ctypes.POINTER(EmitterDesc), _I, _IP],
    "bbg_map_grid": [_P, _IP],
    "bbg_lnm_boundary": [_P, ctypes.c_double, _I, ctypes.c_void_p],
    "bbg_lnm_boundary_single": [_P, ctypes.c_double, _I, ctypes.c_void_p],
    "bbg_lnm_boundary_extended": [_P, ctypes.c_double, _I, _I, ctypes.c_void_p],
    "bbg_lnm_boundary_geometric": [_P, ctypes.c_double, _I, _I, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    "bbg_boundary_test": [_P, _I, ctypes.c_double, ctypes.c_void_p],
    "bbg_energy": [_P, ctypes.c_void_p],
    "bbg_step_host": [_P, ctypes.c_double, _I] + [ctypes.c_void_p] * 8 + [ctypes.c_void_p],
    "bbg_particle_sdf": [_P, _I, ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                         ctypes.c_void_p, ctypes.c_size_t],
    "bbg_collider_set_sdf": [_P, _I, ctypes.POINTER(SdfGrid), ctypes.c_void_p],
    "bbg_collider_generate_sdf": [_P, _I, ctypes.c_double, ctypes.c_double],
    "bbg_collider_get_sdf": [_P, _I, ctypes.POINTER(SdfGrid), ctypes.c_void_p, ctypes.c_size_t,
                             ctypes.POINTER(ctypes.c_size_t)],
    "bbg_mesh_sdf": [_P, ctypes.c_void_p, _I, ctypes.c_void_p, _I, ctypes.c_double, ctypes.c_double,
                     ctypes.POINTER(SdfGrid), ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t), _IP],
    "bbg_collider_set_mesh": [_P, _I, ctypes.c_void_p, _I, ctypes.c_void_p, _I, ctypes.c_double, ctypes.c_double],
    "bbg_marching_cubes": [_P, ctypes.POINTER(SdfGrid), ctypes.c_void_p, ctypes.c_double, _I, ctypes.c_void_p,
                           ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                           ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)],
    "bbg_collider_query": [_P, _I, _I, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    "bbg_map_grid_emit": [_P, ctypes.c_double, ctypes.POINTER(ctypes.c_double), _IP],
    "bbg_checkpoint_save": [_P, ctypes.c_char_p],
    "bbg_checkpoint_load": [_P, ctypes.c_char_p],
    "bbg_checkpoint_write": [_P, ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)],
    "bbg_checkpoint_read": [_P, ctypes.c_char_p, ctypes.c_size_t],
    "bbg_mlp_desc_default": [ctypes.POINTER(MlpDesc)],
    "bbg_mlp_configure": [_P, ctypes.POINTER(MlpDesc)],
    "bbg_mlp_get_params": [_P, _FP],
    "bbg_mlp_set_params": [_P, _FP],
    "bbg_mlp_set_trained": [_P, _I],
    "bbg_mlp_status": [_P, _IP, _IP, _DP],
    "bbg_mlp_infer": [_P, _FP, _I, _FP],
    "bbg_mlp_train_batch": [_P, _FP, _FP, _I],
    "bbg_mlp_get_features": [_P, _FP],
    "bbg_profiler_report": [_P, _I, ctypes.c_char_p, _DP, _IP, _IP,
                            ctypes.POINTER(ctypes.c_int64)],
}
_RES = {"bbg_version": (ctypes.c_char_p, []),
        "bbg_status_string": (ctypes.c_char_p, [_I]),
        "bbg_last_error": (ctypes.c_char_p, [])}

_lib = None


def library_path():
    return _build.lib_path()


def load(build_if_missing=True):
    """Load libbbg.so; builds it in-tree when it is missing or stale."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(path):
        raise ImportError("libbbg.so not found at %s; run bubbles_gb300.build.build()" % path)
    lib = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = ctypes.c_int
        fn.argtypes = args
    for name, (res, args) in _RES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status):
    if status != OK:
        msg = _lib.bbg_last_error().decode() if _lib is not None else ""
        raise BbgError(status, msg)
    return status


def call(name, *args):
    lib = load()
    return check(getattr(lib, name)(*args))


def device_count():
    c = ctypes.c_int(0)
    call("bbg_device_count", ctypes.byref(c))
    return c.value
