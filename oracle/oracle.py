"""ctypes wrapper of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU baseline may import
this module; the product never does.  See sph_oracle.h for what the oracle
restates and how it is pinned.
"""
import ctypes
import os

import numpy as np

from . import build as _build

MAX_COLLIDERS = 16
SHAPE_BOX = 1
SHAPE_SPHERE = 2

POSITION, VELOCITY, FORCE, INTERACTION, DENSITY, PRESSURE = 0, 1, 2, 3, 4, 5
PRED_POSITION, PRED_VELOCITY, PRESSURE_FORCE, PRED_DENSITY = 6, 7, 8, 9
DENSITY_ERROR, SMOOTHED_VELOCITY = 10, 11
VECTOR_FIELDS = {POSITION, VELOCITY, FORCE, INTERACTION, PRED_POSITION, PRED_VELOCITY,
                 PRESSURE_FORCE, SMOOTHED_VELOCITY}

PCISPH_AS_SHIPPED = 0
PCISPH_TOLERANCE = 1
PCISPH_WARM = 2            # warm start, total pressure clamped
PCISPH_WARM_MONOTONE = 3   # warm start, reference (non-negative increment) update
BUCKET = 100


class Shape(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int), ("reverse", ctypes.c_int),
                ("center", ctypes.c_double * 3), ("size", ctypes.c_double * 3),
                ("friction", ctypes.c_double)]


class Params(ctypes.Structure):
    _fields_ = [("eos_exponent", ctypes.c_double),
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
                ("n_colliders", ctypes.c_int),
                ("colliders", Shape * MAX_COLLIDERS),
                ("time_step_limit_scale", ctypes.c_double)]


_LIBS = {}
_D = ctypes.POINTER(ctypes.c_double)
_U32 = ctypes.POINTER(ctypes.c_uint32)
_I32 = ctypes.POINTER(ctypes.c_int32)
_P = ctypes.c_void_p


def _ptr(a, t=_D):
    return a.ctypes.data_as(t)


def load(variant="f32"):
    """Load (building if needed) the FP32 or FP64 oracle library."""
    if variant in _LIBS:
        return _LIBS[variant]
    _build.build()
    lib = ctypes.CDLL(_build.lib_path(variant))
    sig = {
        "orc_float_bytes": (ctypes.c_int, []),
        "orc_set_threads": (None, [ctypes.c_int]),
        "orc_get_threads": (ctypes.c_int, []),
        "orc_create": (_P, [ctypes.POINTER(Params), ctypes.c_int, _D, _D]),
        "orc_destroy": (None, [_P]),
        "orc_scalars": (None, [_P, _D]),
        "orc_grid_info": (None, [_P, _I32, _D]),
        "orc_cell_neighbors": (ctypes.c_int, [_P, ctypes.c_int, _I32]),
        "orc_hash_points": (None, [_P, ctypes.c_int, _D, _U32, _U32]),
        "orc_compute_mass_bcc": (ctypes.c_double, [ctypes.c_double] * 3),
        "orc_compute_delta_denom": (ctypes.c_double, [ctypes.c_double] * 2),
        "orc_build_grid": (ctypes.c_int, [_D, _D, ctypes.c_double, ctypes.c_double, _I32, _D]),
        "orc_kernel_eval": (ctypes.c_double, [ctypes.c_int, ctypes.c_double, ctypes.c_double]),
        "orc_update_grid_distribution": (None, [_P]),
        "orc_compute_particle_interaction": (None, [_P]),
        "orc_compute_density": (None, [_P, ctypes.c_int]),
        "orc_compute_non_pressure_force": (None, [_P]),
        "orc_compute_delta": (ctypes.c_double, [_P, ctypes.c_double]),
        "orc_pressure_force_and_integrate": (ctypes.c_int, [_P, ctypes.c_double, ctypes.c_double,
                                                            ctypes.c_double, ctypes.c_int,
                                                            ctypes.c_int, _D]),
        "orc_time_integration": (None, [_P, ctypes.c_double]),
        "orc_predict_velocity_and_position": (None, [_P, ctypes.c_double, ctypes.c_int]),
        "orc_predict_pressure": (None, [_P, ctypes.c_double]),
        "orc_predict_pressure_force": (None, [_P]),
        "orc_accumulate_and_integrate": (None, [_P, ctypes.c_double]),
        "orc_sph_all_forces": (None, [_P, ctypes.c_double, ctypes.c_int]),
        "orc_pseudo_viscosity": (None, [_P, ctypes.c_double]),
        "orc_number_of_time_steps": (ctypes.c_uint, [_P, ctypes.c_double, ctypes.c_double]),
        "orc_pcisph_substep": (ctypes.c_int, [_P, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                              ctypes.c_int, _D]),
        "orc_sph_substep": (None, [_P, ctypes.c_double, ctypes.c_int]),
        "orc_advance_pcisph": (ctypes.c_int, [_P, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                              ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
        "orc_advance_sph": (ctypes.c_int, [_P, ctypes.c_double, ctypes.c_int]),
        "orc_get_field": (None, [_P, ctypes.c_int, _D]),
        "orc_set_field": (None, [_P, ctypes.c_int, _D]),
        "orc_count": (ctypes.c_int, [_P]),
        "orc_higher_level": (ctypes.c_int, [_P]),
        "orc_set_higher_level": (None, [_P, ctypes.c_int]),
        "orc_get_cells": (ctypes.c_int, [_P, _U32, _U32, _U32]),
        "orc_get_buckets": (ctypes.c_int, [_P, _I32, _I32]),
        "orc_lnm": (None, [_P, ctypes.c_double, ctypes.c_int, _I32]),
        "orc_lnm_single": (None, [_P, ctypes.c_double, ctypes.c_int, _I32]),
        "orc_lnm_extended": (None, [_P, ctypes.c_double, ctypes.c_int, ctypes.c_int, _I32]),
        "orc_lnm_geometric": (None, [_P, ctypes.c_double, ctypes.c_int, ctypes.c_int, _I32, _I32]),
        "orc_xiaowei": (None, [_P, ctypes.c_double, _I32]),
        "orc_dilts": (None, [_P, _I32]),
        "orc_particle_sdf": (ctypes.c_long, [_P, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, _I32,
                                             _I32, _D, _D, ctypes.POINTER(ctypes.c_float), ctypes.c_long]),
        "orc_map_grid": (None, [_P]),
        "orc_map_grid_emit": (ctypes.c_long, [_P, ctypes.c_double, _D, ctypes.c_long]),
        "orc_shape_distance": (None, [ctypes.POINTER(Shape), ctypes.c_int, _D, _D, _I32]),
        "orc_emit_volume": (ctypes.c_long, [ctypes.POINTER(Shape), ctypes.c_int, _D, _D, ctypes.c_double,
                                            ctypes.c_double, _D, ctypes.c_long, _D, _D, ctypes.c_long]),
        "orc_frame_parse": (ctypes.c_long, [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_int),
                                            ctypes.POINTER(ctypes.c_int), _D, _D, _D, _I32, ctypes.c_long]),
        "orc_frame_text": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_int, _D, _D, _D, ctypes.c_double,
                                             ctypes.c_double, ctypes.c_char_p, ctypes.c_size_t]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIBS[variant] = lib
    return lib


def make_params(scene):
    """Params from a scene dict (see bubbles_gb300.scenes for the keys)."""
    p = Params()
    p.eos_exponent = scene.get("eos_exponent", 7.0)
    p.negative_pressure_scale = scene.get("negative_pressure_scale", 0.0)
    p.viscosity = scene.get("viscosity", 0.04)
    p.pseudo_viscosity = scene.get("pseudo_viscosity", 10.0)
    p.sound_speed = scene.get("sound_speed", 100.0)
    p.drag_coefficient = scene.get("drag_coefficient", 1e-4)
    for k in range(3):
        p.gravity[k] = scene.get("gravity", (0.0, -9.8, 0.0))[k]
        p.domain_min[k] = scene["domain_min"][k]
        p.domain_max[k] = scene["domain_max"][k]
    p.target_density = scene.get("target_density", 1000.0)
    p.target_spacing = scene["spacing"]
    p.relative_kernel_radius = scene.get("relative_kernel_radius", 2.0)
    p.mass = scene.get("mass", 0.0) or 0.0
    p.grid_spacing_scale = scene.get("grid_spacing_scale", 2.0)
    cols = scene.get("colliders", [])
    p.n_colliders = len(cols)
    for i, c in enumerate(cols):
        p.colliders[i].type = SHAPE_BOX if c["type"] == "box" else SHAPE_SPHERE
        p.colliders[i].reverse = 1 if c.get("reverse", False) else 0
        for k in range(3):
            p.colliders[i].center[k] = c.get("center", (0, 0, 0))[k]
        if c["type"] == "box":
            for k in range(3):
                p.colliders[i].size[k] = c["size"][k]
        else:
            p.colliders[i].size[0] = c["radius"]
        p.colliders[i].friction = c.get("friction", 0.0)
    p.time_step_limit_scale = scene.get("time_step_limit_scale", 5.0)
    return p


class OracleSim:
    """One oracle simulation (reference semantics; FP32 or FP64)."""

    def __init__(self, scene, pos, vel=None, variant="f32", threads=1):
        self.lib = load(variant)
        self.lib.orc_set_threads(int(threads))
        self.variant = variant
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        self.n = pos.shape[0]
        v = None
        if vel is not None:
            v = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1, 3)
        self._params = make_params(scene)
        self.h = self.lib.orc_create(ctypes.byref(self._params), self.n, _ptr(pos),
                                     _ptr(v) if v is not None else None)
        if not self.h:
            raise RuntimeError("orc_create failed")

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- scalars / grid ---------------------------------------------------
    def scalars(self):
        out = np.zeros(8)
        self.lib.orc_scalars(self.h, _ptr(out))
        keys = ["mass", "kernel_radius", "delta_denom", "mass_over_density_sq",
                "target_spacing", "target_density", "radius", "relative_radius"]
        return dict(zip(keys, out.tolist()))

    def grid_info(self):
        dims = np.zeros(3, np.int32)
        geo = np.zeros(12)
        self.lib.orc_grid_info(self.h, _ptr(dims, _I32), _ptr(geo))
        return dims, geo

    def cell_neighbors(self, cell):
        out = np.zeros(27, np.int32)
        n = self.lib.orc_cell_neighbors(self.h, int(cell), _ptr(out, _I32))
        return out[:n]

    def hash_points(self, pts):
        pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        ids = np.zeros(len(pts), np.uint32)
        uc = np.zeros((len(pts), 3), np.uint32)
        self.lib.orc_hash_points(self.h, len(pts), _ptr(pts), _ptr(ids, _U32), _ptr(uc, _U32))
        return ids, uc

    # --- passes -------------------------------------------------------------
    def update_grid_distribution(self):
        self.lib.orc_update_grid_distribution(self.h)

    def compute_particle_interaction(self):
        self.lib.orc_compute_particle_interaction(self.h)

    def compute_density(self, compute_pressure=1):
        self.lib.orc_compute_density(self.h, int(compute_pressure))

    def compute_non_pressure_force(self):
        self.lib.orc_compute_non_pressure_force(self.h)

    def compute_delta(self, dt):
        return self.lib.orc_compute_delta(self.h, dt)

    def pressure_force_and_integrate(self, dt, max_err, delta, max_it, mode):
        err = ctypes.c_double(0)
        it = self.lib.orc_pressure_force_and_integrate(self.h, dt, max_err, delta, max_it, mode,
                                                       ctypes.byref(err))
        return it, err.value

    def time_integration(self, dt):
        self.lib.orc_time_integration(self.h, dt)

    def predict_velocity_and_position(self, dt, is_first):
        self.lib.orc_predict_velocity_and_position(self.h, dt, int(is_first))

    def predict_pressure(self, delta):
        self.lib.orc_predict_pressure(self.h, delta)

    def predict_pressure_force(self):
        self.lib.orc_predict_pressure_force(self.h)

    def accumulate_and_integrate(self, dt):
        self.lib.orc_accumulate_and_integrate(self.h, dt)

    def sph_all_forces(self, dt, inplace=0):
        self.lib.orc_sph_all_forces(self.h, dt, int(inplace))

    def pseudo_viscosity(self, dt):
        self.lib.orc_pseudo_viscosity(self.h, dt)

    def number_of_time_steps(self, remaining, scale):
        return self.lib.orc_number_of_time_steps(self.h, remaining, scale)

    def pcisph_substep(self, dt, max_err=0.01, max_it=20, mode=PCISPH_TOLERANCE):
        err = ctypes.c_double(0)
        it = self.lib.orc_pcisph_substep(self.h, dt, max_err, max_it, mode, ctypes.byref(err))
        return it, err.value

    def sph_substep(self, dt, inplace=0):
        self.lib.orc_sph_substep(self.h, dt, int(inplace))

    def advance_pcisph(self, dt, max_err=0.01, max_it=20, mode=PCISPH_TOLERANCE):
        iters = ctypes.c_int(0)
        steps = self.lib.orc_advance_pcisph(self.h, dt, max_err, max_it, mode, ctypes.byref(iters))
        return steps, iters.value

    def advance_sph(self, dt, inplace=0):
        return self.lib.orc_advance_sph(self.h, dt, int(inplace))

    # --- fields ---------------------------------------------------------------
    def lnm(self, h, unbounded=False):
        """LNMBoundary's particle levels (1, 2, 0 inside) on the current chains."""
        out = np.zeros(self.n, np.int32)
        self.lib.orc_lnm(self.h, float(h), int(bool(unbounded)), _ptr(out, _I32))
        return out

    def lnm_single(self, h, unbounded=False):
        """LNMBoundarySingle's particle levels (1, 2, 0)."""
        out = np.zeros(self.n, np.int32)
        self.lib.orc_lnm_single(self.h, float(h), int(bool(unbounded)), _ptr(out, _I32))
        return out

    def lnm_extended(self, h, max_level=5, unbounded=False):
        """LNMBoundaryExtended's particle levels (1, 2, 3.. max_level, 0)."""
        out = np.zeros(self.n, np.int32)
        self.lib.orc_lnm_extended(self.h, float(h), int(max_level), int(bool(unbounded)), _ptr(out, _I32))
        return out

    def lnm_geometric(self, h, algorithm, unbounded=False):
        """LNMBoundary with the Xiaowei (1) or Dilts (2) L2 filter: (levels, queued, accepted)."""
        out = np.zeros(self.n, np.int32)
        st = np.zeros(2, np.int32)
        self.lib.orc_lnm_geometric(self.h, float(h), int(algorithm), int(bool(unbounded)),
                                   _ptr(out, _I32), _ptr(st, _I32))
        return out, int(st[0]), int(st[1])

    def xiaowei(self, h):
        """XiaoweiParticleIsBoundary of every particle on the stored densities."""
        out = np.zeros(self.n, np.int32)
        self.lib.orc_xiaowei(self.h, float(h), _ptr(out, _I32))
        return out

    def dilts(self):
        """DiltsSpokeParticleIsBoundary of every particle."""
        out = np.zeros(self.n, np.int32)
        self.lib.orc_dilts(self.h, _ptr(out, _I32))
        return out

    def particle_sdf(self, method, kernel, mc_spacing, resolution=None):
        """The surface app's field (0 Zhu-Bridson, 1 SPH) over the domain grid and the stored
        densities: (nodes, origin float32, spacing float32, values float32, x fastest)."""
        res = np.zeros(3, np.int32) if resolution is None else np.ascontiguousarray(resolution, np.int32)
        nodes = np.zeros(3, np.int32)
        org = np.zeros(3)
        sp = np.zeros(1)
        args = lambda v, cap: (self.h, int(method), float(kernel), float(mc_spacing), int(resolution is not None),
                               _ptr(res, _I32), _ptr(nodes, _I32), _ptr(org), _ptr(sp),
                               v.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), cap)
        total = self.lib.orc_particle_sdf(*args(np.zeros(1, np.float32), 0))
        vals = np.zeros(total, np.float32)
        self.lib.orc_particle_sdf(*args(vals, total))
        return nodes.copy(), org.astype(np.float32), np.float32(sp[0]), vals

    def map_grid(self):
        """ContinuousParticleSetBuilder3::MapGrid on the current chains."""
        self.lib.orc_map_grid(self.h)

    def map_grid_emit(self, distance):
        """Positions MapGridEmit would add (cells ascending, chain order), float64 (k, 3)."""
        k = self.lib.orc_map_grid_emit(self.h, float(distance), None, 0)
        out = np.zeros((max(k, 0), 3))
        self.lib.orc_map_grid_emit(self.h, float(distance), _ptr(out), k)
        return out

    def get(self, field):
        if field in VECTOR_FIELDS:
            out = np.zeros((self.n, 3))
        else:
            out = np.zeros(self.n)
        self.lib.orc_get_field(self.h, field, _ptr(out))
        return out

    def set(self, field, values):
        a = np.ascontiguousarray(values, dtype=np.float64)
        need = self.n * 3 if field in VECTOR_FIELDS else self.n
        if a.size != need:
            raise ValueError("field size mismatch")
        self.lib.orc_set_field(self.h, field, _ptr(a))

    @property
    def higher_level(self):
        return self.lib.orc_higher_level(self.h)

    def set_higher_level(self, v):
        self.lib.orc_set_higher_level(self.h, int(v))

    def cells(self):
        dims, _ = self.grid_info()
        total = int(np.prod(dims))
        cell_of = np.zeros(self.n, np.uint32)
        counts = np.zeros(total, np.uint32)
        chains = np.zeros(self.n, np.uint32)
        self.lib.orc_get_cells(self.h, _ptr(cell_of, _U32), _ptr(counts, _U32), _ptr(chains, _U32))
        return cell_of, counts, chains

    def buckets(self):
        counts = np.zeros(self.n, np.int32)
        ids = np.zeros((self.n, BUCKET), np.int32)
        over = self.lib.orc_get_buckets(self.h, _ptr(counts, _I32), _ptr(ids, _I32))
        return counts, ids, over


def kernel_eval(which, h, r, variant="f32"):
    return load(variant).orc_kernel_eval(which, h, r)


def compute_mass_bcc(density, spacing, kernel_radius, variant="f32"):
    return load(variant).orc_compute_mass_bcc(density, spacing, kernel_radius)


def compute_delta_denom(spacing, kernel_radius, variant="f32"):
    return load(variant).orc_compute_delta_denom(spacing, kernel_radius)


def build_grid(dmin, dmax, spacing, scale, variant="f32"):
    dims = np.zeros(3, np.int32)
    geo = np.zeros(12)
    a = np.asarray(dmin, np.float64)
    b = np.asarray(dmax, np.float64)
    total = load(variant).orc_build_grid(_ptr(a), _ptr(b), spacing, scale, _ptr(dims, _I32),
                                         _ptr(geo))
    return dims, geo, total


def frame_text(pos, vel=None, rho=None, mass=0.0, spacing=0.0, flags=0x01, variant="f32"):
    """SerializerSaveSphDataSet3's frame block for the given state (bytes), as the reference
    prints it: every value rounded to the build's Float, then printf("%g")."""
    lib = load(variant)
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    n = len(pos)
    v = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64).reshape(-1, 3)
    r = None if rho is None else np.ascontiguousarray(rho, dtype=np.float64).reshape(-1)
    args = (n, int(flags), _ptr(pos), _ptr(v) if v is not None else None,
            _ptr(r) if r is not None else None, float(mass), float(spacing))
    need = lib.orc_frame_text(*args, None, 0)
    buf = ctypes.create_string_buffer(need + 1)
    lib.orc_frame_text(*args, buf, need + 1)
    return buf.raw[:need]


def frame_parse(text, flags=0, variant="f32"):
    """SerializerLoadParticles3 restated: (flags, header count, pos, vel, density, boundary)
    of the first fluid section of a frame text; raises ValueError where the reference stops."""
    lib = load(variant)
    cap = text.count(b"\n") + text.count(b"\r") + 1
    pos = np.zeros((cap, 3))
    vel = np.zeros((cap, 3))
    rho = np.zeros(cap)
    bnd = np.zeros(cap, np.int32)
    fl, cnt = ctypes.c_int(flags), ctypes.c_int(0)
    n = lib.orc_frame_parse(text, len(text), ctypes.byref(fl), ctypes.byref(cnt), _ptr(pos), _ptr(vel),
                            _ptr(rho), _ptr(bnd, _I32), cap)
    if n == -1:
        raise ValueError("unknown format letter")
    if n < 0:
        raise ValueError("no complete fluid section")
    return fl.value, cnt.value, pos[:n], vel[:n], rho[:n], bnd[:n]


def emit_volume(shape, spacing, jitter=0.0, velocity=(0.0, 0.0, 0.0), max_particles=2**31 - 1, bounds=None,
                variant="f32", capacity=None):
    """VolumeParticleEmitter3::Emit restated (the caller seeds the C library's rand()):
    (positions, velocities) of the particles emitted in a box or sphere shape dict."""
    lib = load(variant)
    sh = Shape()
    box = shape["type"] == "box"
    sh.type = SHAPE_BOX if box else SHAPE_SPHERE
    sh.reverse = int(bool(shape.get("reverse", False)))
    for k in range(3):
        sh.center[k] = shape.get("center", (0.0, 0.0, 0.0))[k]
        sh.size[k] = shape["size"][k] if box else (shape["radius"] if k == 0 else 0.0)
    bmin = np.array(bounds[0] if bounds else (0, 0, 0), np.float64)
    bmax = np.array(bounds[1] if bounds else (0, 0, 0), np.float64)
    v = np.array(velocity, np.float64)
    if capacity is None:
        capacity = 1 << 22
    pos = np.zeros((capacity, 3))
    vel = np.zeros((capacity, 3))
    n = lib.orc_emit_volume(ctypes.byref(sh), int(bounds is not None), _ptr(bmin), _ptr(bmax), float(spacing),
                            float(jitter), _ptr(v), int(max_particles), _ptr(pos), _ptr(vel), capacity)
    return pos[:min(n, capacity)], vel[:min(n, capacity)]


def shape_distance(shape, points, variant="f32"):
    """Shape::ClosestDistance and IsInside of a box or sphere shape dict at the points."""
    lib = load(variant)
    sh = Shape()
    box = shape["type"] == "box"
    sh.type = SHAPE_BOX if box else SHAPE_SPHERE
    sh.reverse = int(bool(shape.get("reverse", False)))
    for k in range(3):
        sh.center[k] = shape.get("center", (0.0, 0.0, 0.0))[k]
        sh.size[k] = shape["size"][k] if box else (shape["radius"] if k == 0 else 0.0)
    p = np.ascontiguousarray(points, np.float64).reshape(-1, 3)
    d = np.zeros(len(p))
    ins = np.zeros(len(p), np.int32)
    lib.orc_shape_distance(ctypes.byref(sh), len(p), _ptr(p), _ptr(d), _ptr(ins, _I32))
    return d, ins

