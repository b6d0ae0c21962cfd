"""ctypes wrapper of the host-only reference build (oracle/ref) -- test infrastructure.

Only available where the reference checkout exists (the recipe builds from it); used to
pin the CPU oracle and to generate tests/golden/ fixtures.
"""
import ctypes
import os

import numpy as np

from . import oracle as O

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS = {}
_D = ctypes.POINTER(ctypes.c_double)
_U32 = ctypes.POINTER(ctypes.c_uint32)
_I32 = ctypes.POINTER(ctypes.c_int32)
_P = ctypes.c_void_p


def lib_path(variant):
    return os.path.join(_HERE, "_ref", "libbbref_%s.so" % variant)


def available(variant="f32"):
    if os.path.exists(lib_path(variant)):
        return True
    try:
        import importlib.util
        spec = importlib.util.spec_from_file_location("build_ref", os.path.join(_HERE, "ref", "build_ref.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        if mod.available():
            mod.build()
    except Exception:
        return False
    return os.path.exists(lib_path(variant))


def load(variant):
    if variant in _LIBS:
        return _LIBS[variant]
    lib = ctypes.CDLL(lib_path(variant))
    sig = {
        "ref_float_bytes": (ctypes.c_int, []),
        "ref_create": (_P, [ctypes.POINTER(O.Params), ctypes.c_int, _D, _D, ctypes.c_int]),
        "ref_create_continuous": (_P, [ctypes.POINTER(O.Params), ctypes.c_int, _D, _D, ctypes.c_int,
                                       ctypes.c_int]),
        "ref_map_grid": (None, [_P]),
        "ref_generate_collider_sdf": (None, [_P, ctypes.c_int, ctypes.c_double, ctypes.c_double]),
        "ref_make_sdf_sphere_collider": (None, [_P, ctypes.c_int, _D, ctypes.c_double, ctypes.c_double,
                                                ctypes.c_double]),
        "ref_collider_sdf": (ctypes.c_int, [_P, ctypes.c_int, _I32, _D, _D, ctypes.POINTER(ctypes.c_float),
                                            ctypes.c_int]),
        "ref_marching_cubes": (ctypes.c_int, [_I32, _D, _D, ctypes.POINTER(ctypes.c_float), ctypes.c_double,
                                              ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                                              ctypes.POINTER(ctypes.c_float), _I32, ctypes.c_int, ctypes.c_int,
                                              ctypes.POINTER(ctypes.c_int)]),
        "ref_lnm": (None, [_P, ctypes.c_double, ctypes.c_int, _I32]),
        "ref_lnm_single": (None, [_P, ctypes.c_double, ctypes.c_int, _I32]),
        "ref_lnm_extended": (None, [_P, ctypes.c_double, ctypes.c_int, ctypes.c_int, _I32]),
        "ref_lnm_geometric": (None, [_P, ctypes.c_double, ctypes.c_int, ctypes.c_int, _I32, _I32]),
        "ref_xiaowei": (None, [_P, ctypes.c_double, _I32]),
        "ref_dilts": (None, [_P, _I32]),
        "ref_dilts_points": (ctypes.c_int, [ctypes.POINTER(ctypes.c_float), ctypes.c_int]),
        "ref_surface_sdf": (ctypes.c_long, [_D, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_int, _I32, ctypes.c_int, ctypes.c_int, _I32, _D, _D,
                                            ctypes.POINTER(ctypes.c_float), ctypes.c_long, _D,
                                            ctypes.POINTER(ctypes.c_float)]),
        "ref_mesh_sdf": (ctypes.c_int, [_D, ctypes.c_int, _I32, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                        _I32, _D, _D, ctypes.POINTER(ctypes.c_float), ctypes.c_int]),
        "ref_sdf_probe": (None, [_P, ctypes.c_int, ctypes.c_int, _D, _D, _D, _D, _D, _D, _I32]),
        "ref_map_grid_emit": (ctypes.c_int, [_P, ctypes.c_double, _D]),
        "ref_destroy": (None, [_P]),
        "ref_scalars": (None, [_P, _D]),
        "ref_grid_info": (None, [_P, _I32, _D]),
        "ref_update_grid_distribution": (None, [_P]),
        "ref_reset_higher_level": (None, [_P]),
        "ref_higher_level": (ctypes.c_int, [_P]),
        "ref_compute_particle_interaction": (None, [_P]),
        "ref_compute_density": (None, [_P, ctypes.c_int]),
        "ref_compute_non_pressure_force": (None, [_P]),
        "ref_compute_delta": (ctypes.c_double, [_P, ctypes.c_double]),
        "ref_pressure_force_and_integrate": (None, [_P, ctypes.c_double, ctypes.c_double,
                                                    ctypes.c_double, ctypes.c_int]),
        "ref_predict_velocity_and_position": (None, [_P, ctypes.c_double, ctypes.c_int]),
        "ref_predict_pressure": (None, [_P, ctypes.c_double]),
        "ref_predict_pressure_force": (None, [_P]),
        "ref_accumulate_and_integrate": (None, [_P, ctypes.c_double]),
        "ref_pseudo_viscosity": (None, [_P, ctypes.c_double]),
        "ref_time_integration": (None, [_P, ctypes.c_double]),
        "ref_sph_pressure_force": (None, [_P, ctypes.c_double]),
        "ref_number_of_time_steps": (ctypes.c_uint, [_P, ctypes.c_double, ctypes.c_double]),
        "ref_advance_time_step": (None, [_P, ctypes.c_double]),
        "ref_advance": (None, [_P, ctypes.c_double]),
        "ref_get_field": (None, [_P, ctypes.c_int, _D]),
        "ref_set_field": (None, [_P, ctypes.c_int, _D]),
        "ref_get_cells": (ctypes.c_int, [_P, _U32, _U32, _U32]),
        "ref_get_buckets": (None, [_P, _I32, _I32]),
        "ref_save_frame": (None, [_P, ctypes.c_char_p, ctypes.c_int]),
        "ref_emit_volume": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _D, _D, ctypes.c_int, _D, _D, ctypes.c_double,
                                           ctypes.c_double, _D, ctypes.c_int, ctypes.c_uint, _D, _D, ctypes.c_int]),
        "ref_load_frame": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), _D, _D, _D, _I32,
                                          ctypes.c_int]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIBS[variant] = lib
    return lib


class RefSim:
    """One scene built and stepped by the reference's own classes (single thread)."""

    def __init__(self, scene, pos, vel=None, variant="f32", kind=None, continuous=None):
        """continuous: capacity of a ContinuousParticleSetBuilder3 holding the particles
        (MapGrid / MapGridEmit), else a ParticleSetBuilder3 builds the set."""
        self.lib = load(variant)
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        self.n = len(pos)
        v = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64).reshape(-1, 3)
        if kind is None:
            kind = 1 if scene.get("solver", "pcisph") == "sph" else 0
        self._params = O.make_params(scene)
        vp = v.ctypes.data_as(_D) if v is not None else None
        if continuous:
            self.h = self.lib.ref_create_continuous(ctypes.byref(self._params), self.n, pos.ctypes.data_as(_D),
                                                    vp, kind, int(continuous))
        else:
            self.h = self.lib.ref_create(ctypes.byref(self._params), self.n, pos.ctypes.data_as(_D), vp, kind)

    def collider_sdf(self, i):
        """Collider i's field: (nodes, origin, spacing, values float32 x fastest)."""
        nodes = np.zeros(3, np.int32)
        org = np.zeros(3)
        sp = np.zeros(3)
        n = self.lib.ref_collider_sdf(self.h, i, nodes.ctypes.data_as(_I32), org.ctypes.data_as(_D),
                                      sp.ctypes.data_as(_D), None, 0)
        vals = np.zeros(n, np.float32)
        self.lib.ref_collider_sdf(self.h, i, nodes.ctypes.data_as(_I32), org.ctypes.data_as(_D),
                                  sp.ctypes.data_as(_D), vals.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), n)
        return nodes, org, sp, vals

    def sdf_probe(self, i, pts):
        pts = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
        n = len(pts)
        out = {"sample": np.zeros(n), "gradient": np.zeros((n, 3)), "point": np.zeros((n, 3)),
               "normal": np.zeros((n, 3)), "distance": np.zeros(n), "inside": np.zeros(n, np.int32)}
        self.lib.ref_sdf_probe(self.h, i, n, pts.ctypes.data_as(_D), out["sample"].ctypes.data_as(_D),
                               out["gradient"].ctypes.data_as(_D), out["point"].ctypes.data_as(_D),
                               out["normal"].ctypes.data_as(_D), out["distance"].ctypes.data_as(_D),
                               out["inside"].ctypes.data_as(_I32))
        return out

    def lnm(self, h, unbounded=False):
        """LNMBoundary's particle levels (1, 2, 0 inside) on the current chains."""
        out = np.zeros(self.n, np.int32)
        self.lib.ref_lnm(self.h, float(h), int(bool(unbounded)), out.ctypes.data_as(_I32))
        return out

    def lnm_single(self, h, unbounded=False):
        """LNMBoundarySingle's particle levels."""
        out = np.zeros(self.n, np.int32)
        self.lib.ref_lnm_single(self.h, float(h), int(bool(unbounded)), out.ctypes.data_as(_I32))
        return out

    def lnm_extended(self, h, max_level=5, unbounded=False):
        """LNMBoundaryExtended's particle levels."""
        out = np.zeros(self.n, np.int32)
        self.lib.ref_lnm_extended(self.h, float(h), int(max_level), int(bool(unbounded)), out.ctypes.data_as(_I32))
        return out

    def lnm_geometric(self, h, algorithm, unbounded=False):
        """LNMBoundary with the Xiaowei (1) or Dilts (2) L2 filter: (levels, queued, accepted)."""
        out = np.zeros(self.n, np.int32)
        st = np.zeros(2, np.int32)
        self.lib.ref_lnm_geometric(self.h, float(h), int(algorithm), int(bool(unbounded)),
                                   out.ctypes.data_as(_I32), st.ctypes.data_as(_I32))
        return out, int(st[0]), int(st[1])

    def xiaowei(self, h):
        out = np.zeros(self.n, np.int32)
        self.lib.ref_xiaowei(self.h, float(h), out.ctypes.data_as(_I32))
        return out

    def dilts(self):
        out = np.zeros(self.n, np.int32)
        self.lib.ref_dilts(self.h, out.ctypes.data_as(_I32))
        return out

    def map_grid_emit(self, d, velocity=(0.0, 0.0, 0.0)):
        v = np.array(velocity, np.float64)
        self.n = self.lib.ref_map_grid_emit(self.h, float(d), v.ctypes.data_as(_D))
        return self.n

    def __getattr__(self, name):
        fn = getattr(self.lib, "ref_" + name)
        return lambda *a: fn(self.h, *a)

    def get(self, field):
        out = np.zeros((self.n, 3) if field in O.VECTOR_FIELDS else self.n)
        self.lib.ref_get_field(self.h, field, out.ctypes.data_as(_D))
        return out

    def set(self, field, values):
        a = np.ascontiguousarray(values, dtype=np.float64)
        self.lib.ref_set_field(self.h, field, a.ctypes.data_as(_D))

    def scalars_dict(self):
        out = np.zeros(8)
        self.lib.ref_scalars(self.h, out.ctypes.data_as(_D))
        keys = ["mass", "kernel_radius", "delta_denom", "mass_over_density_sq",
                "target_spacing", "target_density", "radius", "relative_radius"]
        return dict(zip(keys, out.tolist()))

    def grid(self):
        dims = np.zeros(3, np.int32)
        geo = np.zeros(12)
        self.lib.ref_grid_info(self.h, dims.ctypes.data_as(_I32), geo.ctypes.data_as(_D))
        return dims, geo

    def cells(self):
        dims, _ = self.grid()
        total = int(np.prod(dims))
        cell_of = np.zeros(self.n, np.uint32)
        counts = np.zeros(total, np.uint32)
        chains = np.zeros(self.n, np.uint32)
        self.lib.ref_get_cells(self.h, cell_of.ctypes.data_as(_U32), counts.ctypes.data_as(_U32),
                               chains.ctypes.data_as(_U32))
        return cell_of, counts, chains

    def frame(self, flags):
        """Bytes SerializerSaveSphDataSet3 appends for the current state."""
        import tempfile
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "frame.txt")
            self.lib.ref_save_frame(self.h, path.encode(), int(flags))
            with open(path, "rb") as f:
                return f.read()

    def buckets(self):
        counts = np.zeros(self.n, np.int32)
        ids = np.zeros((self.n, 100), np.int32)
        self.lib.ref_get_buckets(self.h, counts.ctypes.data_as(_I32), ids.ctypes.data_as(_I32))
        return counts, ids


def load_frame(text, flags=0, variant="f32", capacity=None):
    """SerializerLoadParticles3 of the reference on a frame text: (flags, pos, vel, density,
    boundary) of the first fluid section."""
    import tempfile
    lib = load(variant)
    cap = capacity if capacity is not None else max(16, text.count(b"\n") + text.count(b"\r") + 1)
    pos = np.zeros((cap, 3))
    vel = np.zeros((cap, 3))
    rho = np.zeros(cap)
    bnd = np.zeros(cap, np.int32)
    fl = ctypes.c_int(flags)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "frame.txt")
        with open(path, "wb") as f:
            f.write(text)
        n = lib.ref_load_frame(path.encode(), ctypes.byref(fl), pos.ctypes.data_as(_D), vel.ctypes.data_as(_D),
                               rho.ctypes.data_as(_D), bnd.ctypes.data_as(_I32), cap)
    n = min(n, cap)
    return fl.value, pos[:n], vel[:n], rho[:n], bnd[:n]


def emit_volume(shape, spacing, jitter=0.0, velocity=(0.0, 0.0, 0.0), max_particles=2**31 - 1, seed=1,
                bounds=None, variant="f32", capacity=4 << 20):
    """VolumeParticleEmitter3 of the reference (box or sphere shape dict as in scenes) after
    srand(seed): (positions, velocities) of the emitted particles."""
    lib = load(variant)
    box = shape["type"] == "box"
    center = np.array(shape.get("center", (0.0, 0.0, 0.0)), np.float64)
    size = np.array(shape["size"] if box else (shape["radius"], 0.0, 0.0), np.float64)
    bmin = np.array(bounds[0] if bounds else (0, 0, 0), np.float64)
    bmax = np.array(bounds[1] if bounds else (0, 0, 0), np.float64)
    v = np.array(velocity, np.float64)
    pos = np.zeros((capacity, 3))
    vel = np.zeros((capacity, 3))
    n = lib.ref_emit_volume(1 if box else 2, int(bool(shape.get("reverse", False))), center.ctypes.data_as(_D),
                            size.ctypes.data_as(_D), int(bounds is not None), bmin.ctypes.data_as(_D),
                            bmax.ctypes.data_as(_D), float(spacing), float(jitter), v.ctypes.data_as(_D),
                            int(max_particles), int(seed), pos.ctypes.data_as(_D), vel.ctypes.data_as(_D),
                            capacity)
    return pos[:min(n, capacity)], vel[:min(n, capacity)]


def mesh_sdf(vertices, triangles, dx, margin, variant="f32"):
    """MakeMesh + GenerateShapeSDF of the reference: (nodes, origin, spacing, values)."""
    lib = load(variant)
    v = np.ascontiguousarray(vertices, np.float64).reshape(-1, 3)
    t = np.ascontiguousarray(triangles, np.int32).reshape(-1, 3)
    nodes = np.zeros(3, np.int32)
    org = np.zeros(3)
    sp = np.zeros(3)
    args = (v.ctypes.data_as(_D), len(v), t.ctypes.data_as(_I32), len(t), float(dx), float(margin),
            nodes.ctypes.data_as(_I32), org.ctypes.data_as(_D), sp.ctypes.data_as(_D))
    n = lib.ref_mesh_sdf(*args, None, 0)
    vals = np.zeros(n, np.float32)
    lib.ref_mesh_sdf(*args, vals.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), n)
    return nodes, org, sp, vals


def surface_sdf(pos, spacing, kernel, mc_spacing, method=0, resolution=None, direct=False, variant="f32"):
    """The surface app's particle-to-field step (ParticlesToSDF_Surface; method 0 Zhu-Bridson,
    1 SPH): dict of nodes, origin, spacing, values (x fastest) and, unless direct, the domain
    grid's bounds and the particles' densities."""
    lib = load(variant)
    p = np.ascontiguousarray(pos, np.float64)
    n = len(p)
    res = np.zeros(3, np.int32) if resolution is None else np.ascontiguousarray(resolution, np.int32)
    nodes = np.zeros(3, np.int32)
    org = np.zeros(3)
    sp = np.zeros(1)
    dom = np.zeros(6)
    dens = np.zeros(max(n, 1), np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    args = lambda vals, cap: (p.ctypes.data_as(_D), n, float(spacing), float(kernel), float(mc_spacing),
                              int(resolution is not None), res.ctypes.data_as(_I32), int(method), int(bool(direct)),
                              nodes.ctypes.data_as(_I32), org.ctypes.data_as(_D), sp.ctypes.data_as(_D),
                              vals.ctypes.data_as(fp), cap, dom.ctypes.data_as(_D), dens.ctypes.data_as(fp))
    total = lib.ref_surface_sdf(*args(np.zeros(1, np.float32), 0))
    vals = np.zeros(total, np.float32)
    lib.ref_surface_sdf(*args(vals, total))
    out = {"nodes": nodes.copy(), "origin": org.astype(np.float32), "spacing": np.float32(sp[0]), "values": vals}
    if not direct:
        out["domain"] = dom.astype(np.float32)
        out["density"] = dens[:n].copy()
    return out


def dilts_points(variant="f32"):
    """DiltsSpokeTakeUniformPoint's points around the origin for r = 1, (k, 3) float32."""
    lib = load(variant)
    out = np.zeros((5000, 3), np.float32)
    k = lib.ref_dilts_points(out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), 5000)
    return out[:k]


def marching_cubes(nodes, origin, spacing, values, iso=0.0, rotate=False, variant="f32"):
    """MarchingCubes of the reference (single thread): (points, normals, triangles)."""
    lib = load(variant)
    nodes = np.ascontiguousarray(nodes, np.int32)
    org = np.ascontiguousarray(origin, np.float64)
    sp = np.ascontiguousarray(spacing, np.float64)
    vals = np.ascontiguousarray(values, np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    nt = ctypes.c_int()
    cap = 12 * int(np.prod(nodes))
    pts = np.zeros((cap, 3), np.float32)
    nrm = np.zeros((cap, 3), np.float32)
    tri = np.zeros((cap, 3), np.int32)
    n = lib.ref_marching_cubes(nodes.ctypes.data_as(_I32), org.ctypes.data_as(_D), sp.ctypes.data_as(_D),
                               vals.ctypes.data_as(fp), float(iso), int(bool(rotate)), pts.ctypes.data_as(fp),
                               nrm.ctypes.data_as(fp), tri.ctypes.data_as(_I32), cap, cap, ctypes.byref(nt))
    return pts[:n], nrm[:n], tri[:nt.value]

