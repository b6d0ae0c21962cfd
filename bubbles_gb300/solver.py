"""Python mirror of the reference solver API over the bbg C ABI.

`PciSphSolver3` and `SphSolver3` keep the reference's method names
(src/core/pcisph_solver.h:56-83, src/core/sph_solver.h:76-96) and free-function
passes (src/core/sph_solver.h:124-196, src/core/pcisph_solver.h:85-99).  Host arrays
are numpy float32 (n, 3) / (n,); device variants take torch CUDA tensors.  Every
failure raises `BbgError` -- there is no CPU path.
"""
import ctypes

import numpy as np

from . import _native as N


def _fptr(a):
    return a.ctypes.data_as(N._FP)


def desc_from_scene(scene, device=0):
    """bbg_solver_desc from a scene dict (see bubbles_gb300.scenes)."""
    d = N.SolverDesc()
    kind = N.SOLVER_SPH if scene.get("solver", "pcisph") == "sph" else N.SOLVER_PCISPH
    N.call("bbg_solver_desc_default", ctypes.byref(d), kind)
    for key in ("eos_exponent", "negative_pressure_scale", "viscosity", "pseudo_viscosity",
                "sound_speed", "drag_coefficient", "target_density", "relative_kernel_radius",
                "grid_spacing_scale", "time_step_limit_scale", "max_density_error_ratio"):
        if key in scene:
            setattr(d, key, float(scene[key]))
    d.target_spacing = float(scene["spacing"])
    d.mass = float(scene.get("mass", 0.0) or 0.0)
    if "gravity" in scene:
        for k in range(3):
            d.gravity[k] = float(scene["gravity"][k])
    for k in range(3):
        d.domain_min[k] = float(scene["domain_min"][k])
        d.domain_max[k] = float(scene["domain_max"][k])
    mode = scene.get("pcisph_mode", "tolerance")
    d.pcisph_mode = N.PCISPH_TOLERANCE if mode == "tolerance" else N.PCISPH_AS_SHIPPED
    d.max_iterations = int(scene.get("max_iterations", 20 if mode == "tolerance" else 5))
    d.device = int(device)
    d.pressure_init = {"zero": 0, "previous": 1, "learned": 2}[scene.get("pressure_init", "zero")]
    d.warm_rule = {"clamp_total": 0, "monotone": 1}[scene.get("warm_rule", "monotone")]
    d.warm_scale = float(scene.get("warm_scale", 0.0))
    return d


def fill_shape(dst, c):
    """A bbg_shape from a shape dict ({"type": "box", "size", "center", "reverse"} or
    {"type": "sphere", "radius", ...})."""
    dst.type = {"box": N.SHAPE_BOX, "sphere": N.SHAPE_SPHERE, "sdf": N.SHAPE_SDF}[c["type"]]
    dst.reverse = 1 if c.get("reverse", False) else 0
    for k in range(3):
        dst.center[k] = float(c.get("center", (0.0, 0.0, 0.0))[k])
    if c["type"] == "box":
        for k in range(3):
            dst.size[k] = float(c["size"][k])
    elif c["type"] == "sphere":
        dst.size[0] = float(c["radius"])
    dst.friction = float(c.get("friction", 0.0))


def shapes_from_scene(scene):
    cols = scene.get("colliders", [])
    arr = (N.Shape * max(1, len(cols)))()
    for i, c in enumerate(cols):
        fill_shape(arr[i], c)
    return arr, len(cols)


BOUNDARY_TESTS = {"xiaowei": 1, "dilts": 2}
SURFACE_METHODS = {"zhu": 0, "sph": 1}


def surface_scene(pos, spacing):
    """The surface app's SPH set and domain for particles at `spacing`
    (UtilBuildGridForBuilder: the positions' float bounds grown by the spacing, cells of
    twice the spacing; SphSolver3::Setup with relative kernel radius 2, mass from
    ComputeMass)."""
    p = np.asarray(pos, np.float32).reshape(-1, 3)
    sp = np.float32(spacing)
    lo = p.min(axis=0) - sp
    hi = p.max(axis=0) + sp
    return {"solver": "sph", "spacing": float(spacing), "target_density": 1000.0, "relative_kernel_radius": 2.0,
            "grid_spacing_scale": 2.0, "domain_min": tuple(float(x) for x in lo),
            "domain_max": tuple(float(x) for x in hi), "colliders": [], "gravity": (0.0, 0.0, 0.0)}


def reconstruct_surface(pos, spacing, kernel_radius, mc_spacing, method="zhu", iso=None, resolution=None,
                        device=0):
    """The reference's surface app on the device: particles -> field (Zhu-Bridson or SPH,
    densities from the set's own density pass) -> MarchingCubes at iso (0 by default).
    Returns (points, normals, triangles)."""
    sc = surface_scene(pos, spacing)
    with Solver(sc, pos=pos, device=device) as s:
        s.update_grid_distribution()
        s.compute_density(0)
        nodes, org, sp, vals = s.particle_sdf(method, kernel_radius, mc_spacing, resolution)
        return s.marching_cubes(nodes, org, sp, vals, 0.0 if iso is None else iso)


class Solver:
    """One GPU particle system (PciSphSolver3 or SphSolver3 semantics)."""

    def __init__(self, scene, capacity=None, device=0, pos=None, vel=None, setup=True):
        self.scene = scene
        self.desc = desc_from_scene(scene, device)
        n = capacity if capacity is not None else (len(pos) if pos is not None else 0)
        if n <= 0:
            raise ValueError("need a capacity or initial positions")
        h = ctypes.c_void_p()
        N.call("bbg_create", ctypes.byref(self.desc), int(n), ctypes.byref(h))
        self.h = h
        shapes, count = shapes_from_scene(scene)
        N.call("bbg_set_colliders", self.h, shapes, count)
        self.n = 0
        if scene.get("pressure_init") == "learned" and scene.get("mlp"):
            self.mlp_configure(**scene["mlp"])
        if pos is not None:
            self.upload(pos, vel)
            if setup:
                self.setup()

    # lifetime ---------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None) and self.h.value:
            N.load().bbg_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # particles ---------------------------------------------------------------
    def upload(self, pos, vel=None):
        p = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
        v = None if vel is None else np.ascontiguousarray(vel, dtype=np.float32).reshape(-1, 3)
        N.call("bbg_upload_particles", self.h, _fptr(p), _fptr(v) if v is not None else None,
               int(p.shape[0]))
        self.n = int(p.shape[0])

    def upload_device(self, pos, vel=None):
        """pos/vel: contiguous float32 CUDA tensors of shape (n, 3)."""
        n = int(pos.shape[0])
        N.call("bbg_upload_particles_device", self.h, ctypes.c_void_p(pos.data_ptr()),
               ctypes.c_void_p(vel.data_ptr()) if vel is not None else None, n)
        self.n = n

    def setup(self):
        N.call("bbg_setup", self.h)

    def emit_volume(self, shape, spacing, jitter=0.0, velocity=(0.0, 0.0, 0.0), max_particles=None,
                    bounds=None, append=False):
        """VolumeParticleEmitter3 of a box or sphere shape dict on the device (the jitter uses
        the C library's rand(), seeded by the caller); returns how many particles were
        emitted.  append=False replaces the particles, True adds them after the existing."""
        e = N.EmitterDesc()
        N.call("bbg_emitter_desc_default", ctypes.byref(e))
        fill_shape(e.shape, shape)
        if bounds is not None:
            e.use_bounds = 1
            for k in range(3):
                e.bounds_min[k] = float(bounds[0][k])
                e.bounds_max[k] = float(bounds[1][k])
        e.spacing = float(spacing)
        e.jitter = float(jitter)
        for k in range(3):
            e.initial_velocity[k] = float(velocity[k])
        if max_particles is not None:
            e.max_particles = int(max_particles)
        out = ctypes.c_int()
        N.call("bbg_emit_volume", self.h, ctypes.byref(e), int(bool(append)), ctypes.byref(out))
        self.n = self.particle_count()
        return out.value

    # --- colliders with signed-distance fields -------------------------------------
    def set_sdf(self, index, nodes, origin, spacing, values, bounds=None):
        """Attach a vertex-centred field (nodes per axis, x fastest values) to collider
        `index`; bounds=(lo, hi) marks a mesh's field."""
        g = N.SdfGrid()
        for k in range(3):
            g.nodes[k] = int(nodes[k])
            g.origin[k] = float(origin[k])
            g.spacing[k] = float(spacing[k] if np.ndim(spacing) else spacing)
        if bounds is not None:
            g.bounded = 1
            for k in range(3):
                g.bounds_min[k] = float(bounds[0][k])
                g.bounds_max[k] = float(bounds[1][k])
        v = np.ascontiguousarray(values, dtype=np.float32).reshape(-1)
        if v.size != int(np.prod([int(x) for x in nodes])):
            raise ValueError("values must hold one float per node")
        N.call("bbg_collider_set_sdf", self.h, int(index), ctypes.byref(g), v.ctypes.data)

    def generate_sdf(self, index, dx=0.01, margin=0.1):
        """GenerateShapeSDF of a box or sphere collider on the device (attached to it)."""
        N.call("bbg_collider_generate_sdf", self.h, int(index), float(dx), float(margin))

    def mesh_sdf(self, vertices, triangles, dx=0.01, margin=0.1):
        """GenerateShapeSDF of a triangle mesh on the device: (nodes, origin, spacing, values,
        bounds, stuck rays)."""
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(triangles, dtype=np.int32).reshape(-1, 3)
        g = N.SdfGrid()
        cnt = ctypes.c_size_t()
        stuck = ctypes.c_int()
        args = (self.h, v.ctypes.data, len(v), t.ctypes.data, len(t), float(dx), float(margin), ctypes.byref(g))
        N.call("bbg_mesh_sdf", *args, None, 0, ctypes.byref(cnt), ctypes.byref(stuck))
        vals = np.empty(cnt.value, np.float32)
        N.call("bbg_mesh_sdf", *args, vals.ctypes.data, vals.size, ctypes.byref(cnt), ctypes.byref(stuck))
        return (np.array(g.nodes[:]), np.array(g.origin[:]), np.array(g.spacing[:]), vals,
                (np.array(g.bounds_min[:]), np.array(g.bounds_max[:])), stuck.value)

    def set_mesh_collider(self, index, vertices, triangles, dx=0.01, margin=0.1):
        """A field-only collider `index` becomes the mesh (its field generated on the device)."""
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(triangles, dtype=np.int32).reshape(-1, 3)
        N.call("bbg_collider_set_mesh", self.h, int(index), v.ctypes.data, len(v), t.ctypes.data, len(t),
               float(dx), float(margin))

    def get_sdf(self, index):
        """(nodes, origin, spacing, values) of collider `index`'s field."""
        g = N.SdfGrid()
        cnt = ctypes.c_size_t()
        N.call("bbg_collider_get_sdf", self.h, int(index), ctypes.byref(g), None, 0, ctypes.byref(cnt))
        vals = np.empty(cnt.value, np.float32)
        N.call("bbg_collider_get_sdf", self.h, int(index), ctypes.byref(g), vals.ctypes.data, vals.size,
               ctypes.byref(cnt))
        return np.array(g.nodes[:]), np.array(g.origin[:]), np.array(g.spacing[:]), vals

    def collider_query(self, index, points):
        """Collider `index` at the points as the collision code sees it: dict of sample,
        gradient, point, normal, distance, inside."""
        p = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
        n = len(p)
        out = {"sample": np.zeros(n, np.float32), "gradient": np.zeros((n, 3), np.float32),
               "point": np.zeros((n, 3), np.float32), "normal": np.zeros((n, 3), np.float32),
               "distance": np.zeros(n, np.float32), "inside": np.zeros(n, np.int32)}
        N.call("bbg_collider_query", self.h, int(index), n, p.ctypes.data, out["sample"].ctypes.data,
               out["gradient"].ctypes.data, out["point"].ctypes.data, out["normal"].ctypes.data,
               out["distance"].ctypes.data, out["inside"].ctypes.data)
        return out

    def step_host(self, dt, pos, vel, pressure=None, divergence=None, pos_out=None, vel_out=None,
                  pressure_out=None, divergence_out=None):
        """One substep with the state in host arrays (float32, caller order): upload, advance,
        download into the given outputs, one synchronisation (bbg_step_host)."""
        def ptr(a, shape):
            if a is None:
                return None
            assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"] and a.size == int(np.prod(shape))
            return a.ctypes.data
        n = int(np.asarray(pos).shape[0])
        N.call("bbg_step_host", self.h, float(dt), n, ptr(pos, (n, 3)), ptr(vel, (n, 3)), ptr(pressure, (n,)),
               ptr(divergence, (n,)), ptr(pos_out, (n, 3)), ptr(vel_out, (n, 3)), ptr(pressure_out, (n,)),
               ptr(divergence_out, (n,)), None)
        self.n = n

    def energy(self):
        """FP64 totals of the state: mass, kinetic, potential, momentum (3)."""
        out = np.zeros(6)
        N.call("bbg_energy", self.h, out.ctypes.data)
        return {"mass": out[0], "kinetic": out[1], "potential": out[2], "momentum": out[3:6].copy()}

    def particle_sdf(self, method="zhu", kernel_radius=0.04, mc_spacing=0.02, resolution=None):
        """ParticlesToSDF_Surface's field over this solver's domain ("zhu" Zhu-Bridson, "sph"):
        (nodes, origin, spacing, values), values x fastest."""
        m = SURFACE_METHODS.get(method, method)
        g = N.SdfGrid()
        res = None if resolution is None else (ctypes.c_int * 3)(*[int(r) for r in resolution])
        N.call("bbg_particle_sdf", self.h, int(m), float(kernel_radius), float(mc_spacing), res, ctypes.byref(g),
               None, 0)
        vals = np.empty(int(np.prod(g.nodes[:])), np.float32)
        N.call("bbg_particle_sdf", self.h, int(m), float(kernel_radius), float(mc_spacing), res, ctypes.byref(g),
               vals.ctypes.data, vals.size)
        return np.array(g.nodes[:]), np.array(g.origin[:]), np.array(g.spacing[:]), vals

    def marching_cubes(self, nodes, origin, spacing, values, iso=0.0, rotate_faces=False):
        """MarchingCubes of a vertex-centred field on the device: (points, normals,
        triangles)."""
        g = N.SdfGrid()
        for k in range(3):
            g.nodes[k] = int(nodes[k])
            g.origin[k] = float(origin[k])
            g.spacing[k] = float(spacing[k] if np.ndim(spacing) else spacing)
        v = np.ascontiguousarray(values, dtype=np.float32).reshape(-1)
        npt, ntr = ctypes.c_size_t(), ctypes.c_size_t()
        st = N.load().bbg_marching_cubes(self.h, ctypes.byref(g), v.ctypes.data, float(iso), int(bool(rotate_faces)),
                                         None, None, 0, None, 0, ctypes.byref(npt), ctypes.byref(ntr))
        if st not in (N.OK, 4):
            N.call("bbg_marching_cubes", self.h, ctypes.byref(g), v.ctypes.data, float(iso), 0, None, None, 0,
                   None, 0, ctypes.byref(npt), ctypes.byref(ntr))
        pts = np.empty((npt.value, 3), np.float32)
        nrm = np.empty((npt.value, 3), np.float32)
        tri = np.empty((ntr.value, 3), np.int32)
        N.call("bbg_marching_cubes", self.h, ctypes.byref(g), v.ctypes.data, float(iso), int(bool(rotate_faces)),
               pts.ctypes.data, nrm.ctypes.data, npt.value, tri.ctypes.data, ntr.value, ctypes.byref(npt),
               ctypes.byref(ntr))
        return pts, nrm, tri

    def lnm_boundary(self, h, unbounded=False):
        """LNMBoundary: each particle's level (1, 2, 0 inside), caller order."""
        out = np.zeros(self.n, np.int32)
        N.call("bbg_lnm_boundary", self.h, float(h), int(bool(unbounded)), out.ctypes.data)
        return out

    def lnm_boundary_single(self, h, unbounded=False):
        """LNMBoundarySingle: the N2x2 classification in one pass (1, 2, 0), caller order."""
        out = np.zeros(self.n, np.int32)
        N.call("bbg_lnm_boundary_single", self.h, float(h), int(bool(unbounded)), out.ctypes.data)
        return out

    def lnm_boundary_extended(self, h, max_level=5, unbounded=False):
        """LNMBoundaryExtended: levels 1, 2 (filtered L2), 3.. max_level, 0, caller order."""
        out = np.zeros(self.n, np.int32)
        N.call("bbg_lnm_boundary_extended", self.h, float(h), int(max_level), int(bool(unbounded)),
               out.ctypes.data)
        return out

    def lnm_boundary_geometric(self, h, algorithm, unbounded=False):
        """LNMBoundary with the Xiaowei ("xiaowei" / 1) or Dilts ("dilts" / 2) L2 filter:
        (levels, queued, accepted)."""
        alg = BOUNDARY_TESTS.get(algorithm, algorithm)
        out = np.zeros(self.n, np.int32)
        q, a = ctypes.c_int(), ctypes.c_int()
        N.call("bbg_lnm_boundary_geometric", self.h, float(h), int(alg), int(bool(unbounded)), out.ctypes.data,
               ctypes.byref(q), ctypes.byref(a))
        return out, q.value, a.value

    def boundary_test(self, method, h=0.0):
        """XiaoweiBoundary ("xiaowei", at h) or DiltsSpokeBoundary ("dilts"): 1 per boundary particle."""
        out = np.zeros(self.n, np.int32)
        N.call("bbg_boundary_test", self.h, int(BOUNDARY_TESTS.get(method, method)), float(h), out.ctypes.data)
        return out

    def map_grid(self):
        """ContinuousParticleSetBuilder3::MapGrid: remember the occupied cells' positions."""
        out = ctypes.c_int()
        N.call("bbg_map_grid", self.h, ctypes.byref(out))
        return out.value

    def map_grid_emit(self, distance, velocity=(0.0, 0.0, 0.0)):
        """ContinuousParticleSetBuilder3::MapGridEmit: refill the mapped cells; returns how
        many particles were added."""
        v = (ctypes.c_double * 3)(*[float(x) for x in velocity])
        out = ctypes.c_int()
        N.call("bbg_map_grid_emit", self.h, float(distance), v, ctypes.byref(out))
        self.n = self.particle_count()
        return out.value

    def particle_count(self):
        n = ctypes.c_int()
        N.call("bbg_particle_count", self.h, ctypes.byref(n))
        return n.value

    def set_colliders(self, colliders):
        scene = dict(self.scene, colliders=colliders)
        shapes, count = shapes_from_scene(scene)
        N.call("bbg_set_colliders", self.h, shapes, count)

    def set_stream(self, stream):
        """stream: a torch.cuda.Stream (or None for the solver's own stream)."""
        N.call("bbg_set_stream", self.h, ctypes.c_void_p(stream.cuda_stream) if stream else None)

    def synchronize(self):
        N.call("bbg_synchronize", self.h)

    # stepping ----------------------------------------------------------------
    def advance(self, dt):
        st = N.StepStats()
        N.call("bbg_advance", self.h, float(dt), ctypes.byref(st))
        return st.as_dict()

    def advance_time_step(self, dt, stats=False):
        if not stats:
            N.call("bbg_advance_time_step", self.h, float(dt), None)
            return None
        st = N.StepStats()
        N.call("bbg_advance_time_step", self.h, float(dt), ctypes.byref(st))
        return st.as_dict()

    def stats(self):
        st = N.StepStats()
        N.call("bbg_get_stats", self.h, ctypes.byref(st))
        return st.as_dict()

    # passes --------------------------------------------------------------------
    def update_grid_distribution(self):
        N.call("bbg_update_grid_distribution", self.h)

    def compute_particle_interaction(self):
        N.call("bbg_compute_particle_interaction", self.h)

    def compute_density(self, compute_pressure=1):
        N.call("bbg_compute_density", self.h, int(compute_pressure))

    def compute_non_pressure_force(self):
        N.call("bbg_compute_non_pressure_force", self.h)

    def compute_pressure_force(self, dt):
        N.call("bbg_compute_pressure_force", self.h, float(dt))

    def time_integration(self, dt):
        N.call("bbg_time_integration", self.h, float(dt))

    def compute_pseudo_viscosity_interpolation(self, dt):
        N.call("bbg_compute_pseudo_viscosity_interpolation", self.h, float(dt))

    def compute_pressure_force_and_integrate(self, dt, max_err, delta, max_it):
        st = N.StepStats()
        N.call("bbg_compute_pressure_force_and_integrate", self.h, float(dt), float(max_err),
               float(delta), int(max_it), ctypes.byref(st))
        return st.as_dict()

    def predict_velocity_and_position(self, dt, is_first):
        N.call("bbg_predict_velocity_and_position", self.h, float(dt), int(is_first))

    def predict_pressure(self, delta):
        N.call("bbg_predict_pressure", self.h, float(delta))

    def predict_pressure_force(self):
        N.call("bbg_predict_pressure_force", self.h)

    def accumulate_and_integrate(self, dt):
        N.call("bbg_accumulate_and_integrate", self.h, float(dt))

    def compute_delta(self, dt):
        d = ctypes.c_double()
        N.call("bbg_compute_delta", self.h, float(dt), ctypes.byref(d))
        return d.value

    def compute_number_of_time_steps(self, remaining, scale):
        c = ctypes.c_uint()
        N.call("bbg_compute_number_of_time_steps", self.h, float(remaining), float(scale),
               ctypes.byref(c))
        return c.value

    # state ---------------------------------------------------------------------
    def get(self, field, out=None):
        shape = (self.n, 3) if field in N.VECTOR_FIELDS else (self.n,)
        if out is None:
            out = np.zeros(shape, np.float32)
        elif out.dtype != np.float32 or not out.flags.c_contiguous or out.size != int(np.prod(shape)):
            raise ValueError("field buffer must be contiguous float32 of shape %s" % (shape,))
        N.call("bbg_get_field", self.h, int(field), _fptr(out))
        return out

    def set(self, field, values):
        shape = (self.n, 3) if field in N.VECTOR_FIELDS else (self.n,)
        a = np.ascontiguousarray(values, dtype=np.float32).reshape(shape)
        N.call("bbg_set_field", self.h, int(field), _fptr(a))

    def download(self, out_pos=None, out_vel=None):
        """Positions and velocities in the caller's particle order (float32 (n, 3))."""
        p = out_pos if out_pos is not None else np.zeros((self.n, 3), np.float32)
        v = out_vel if out_vel is not None else np.zeros((self.n, 3), np.float32)
        for a in (p, v):
            if a.dtype != np.float32 or not a.flags.c_contiguous or a.size != 3 * self.n:
                raise ValueError("download buffers must be contiguous float32 (n, 3)")
        N.call("bbg_download", self.h, _fptr(p), _fptr(v))
        return p, v

    def download_device(self, pos, vel):
        N.call("bbg_download_device", self.h, ctypes.c_void_p(pos.data_ptr()),
               ctypes.c_void_p(vel.data_ptr()))

    def scalars(self):
        out = (ctypes.c_double * 8)()
        N.call("bbg_get_scalars", self.h, out)
        keys = ["mass", "kernel_radius", "delta_denom", "mass_over_density_sq",
                "target_spacing", "target_density", "radius", "relative_radius"]
        return dict(zip(keys, list(out)))

    def grid(self):
        dims = (ctypes.c_int * 3)()
        geo = (ctypes.c_double * 12)()
        N.call("bbg_get_grid", self.h, dims, geo)
        return np.array(list(dims), np.int32), np.array(list(geo))

    def dump_grid(self):
        dims, _ = self.grid()
        total = int(np.prod(dims))
        cell_of = np.zeros(self.n, np.uint32)
        counts = np.zeros(total, np.uint32)
        ids = np.zeros(self.n, np.uint32)
        N.call("bbg_dump_grid", self.h, cell_of.ctypes.data_as(N._UP),
               counts.ctypes.data_as(N._UP), ids.ctypes.data_as(N._UP))
        return cell_of, counts, ids

    def use_cuda_graphs(self, on=True):
        N.call("bbg_use_cuda_graphs", self.h, int(bool(on)))

    def profiler_enable(self, on=True):
        N.call("bbg_profiler_enable", self.h, int(bool(on)))

    def profiler_report(self):
        """{kernel: (total_ms, launches that did work)}, total kernel launches."""
        m = 32
        names = ctypes.create_string_buffer(32 * m)
        ms = (ctypes.c_double * m)()
        cnt = (ctypes.c_int * m)()
        k = ctypes.c_int()
        total = ctypes.c_int64()
        N.call("bbg_profiler_report", self.h, m, names, ms, cnt, ctypes.byref(k), ctypes.byref(total))
        out = {}
        for i in range(k.value):
            name = names.raw[32 * i:32 * i + 32].split(b"\0", 1)[0].decode()
            out[name] = (ms[i], cnt[i])
        return out, total.value

    # --- particle frames (reference text format) ------------------------------------
    def frame_text(self, flags=N.FRAME_POSITION, out=None):
        """The SerializerSaveSphDataSet3 block of the current state, as bytes; with `out`
        (a writable buffer such as a bytearray) it is written there and its length returned."""
        need = ctypes.c_size_t()
        if out is not None:
            buf = np.frombuffer(out, dtype=np.uint8)
            N.call("bbg_frame_text", self.h, int(flags), buf.ctypes.data, buf.nbytes, ctypes.byref(need))
            return need.value
        st = N.load().bbg_frame_text(self.h, int(flags), None, 0, ctypes.byref(need))
        if st not in (N.OK, 4):   # 4: capacity (size query)
            N.call("bbg_frame_text", self.h, int(flags), None, 0, ctypes.byref(need))
        buf = np.empty(need.value, np.uint8)
        N.call("bbg_frame_text", self.h, int(flags), buf.ctypes.data, buf.nbytes, ctypes.byref(need))
        return buf.tobytes()

    def frame_append(self, path, flags=N.FRAME_POSITION):
        N.call("bbg_frame_append", self.h, int(flags), str(path).encode())

    def frame_load(self, source, flags=0):
        """SerializerLoadSphDataSet3: the first fluid section of a frame (a path, or the
        frame's bytes) becomes this solver's particles; returns the section's flags."""
        fl = ctypes.c_int(int(flags))
        if isinstance(source, (bytes, bytearray)):
            N.call("bbg_frame_load_text", self.h, bytes(source), len(source), ctypes.byref(fl))
        else:
            N.call("bbg_frame_load", self.h, str(source).encode(), ctypes.byref(fl))
        self.n = self.particle_count()
        return fl.value

    # --- checkpoint (exact resume) ----------------------------------------------
    def checkpoint(self):
        """The solver state as checkpoint bytes (bbg_checkpoint_write)."""
        need = ctypes.c_size_t()
        st = N.load().bbg_checkpoint_write(self.h, None, 0, ctypes.byref(need))
        if st not in (N.OK, 4):   # 4: capacity (size query)
            N.call("bbg_checkpoint_write", self.h, None, 0, ctypes.byref(need))
        buf = ctypes.create_string_buffer(need.value)
        N.call("bbg_checkpoint_write", self.h, buf, need.value, ctypes.byref(need))
        return buf.raw[:need.value]

    def restore(self, data):
        """Continue from checkpoint bytes written by a solver with the same description."""
        N.call("bbg_checkpoint_read", self.h, bytes(data), len(data))
        self.n = self.particle_count()

    def save_checkpoint(self, path):
        N.call("bbg_checkpoint_save", self.h, str(path).encode())

    def load_checkpoint(self, path):
        N.call("bbg_checkpoint_load", self.h, str(path).encode())
        self.n = self.particle_count()

    # --- launch tuning ----------------------------------------------------------
    def tuning(self):
        t = N.Tuning()
        N.call("bbg_get_tuning", self.h, ctypes.byref(t))
        return {name: getattr(t, name) for name, _ in t._fields_}

    def set_tuning(self, **values):
        t = N.Tuning()
        N.call("bbg_get_tuning", self.h, ctypes.byref(t))
        for k, v in values.items():
            setattr(t, k, int(v))
        N.call("bbg_set_tuning", self.h, ctypes.byref(t))

    # --- learned warm start ----------------------------------------------------
    def mlp_configure(self, **settings):
        """(Re)initialise the warm-start MLP; settings override bbg_mlp_desc_default."""
        d = N.MlpDesc()
        N.call("bbg_mlp_desc_default", ctypes.byref(d))
        for k, v in settings.items():
            setattr(d, k, v)
        N.call("bbg_mlp_configure", self.h, ctypes.byref(d))

    def mlp_params(self):
        out = np.zeros(N.MLP_PARAMS, np.float32)
        N.call("bbg_mlp_get_params", self.h, _fptr(out))
        return out

    def mlp_set_params(self, theta):
        a = np.ascontiguousarray(theta, dtype=np.float32).reshape(N.MLP_PARAMS)
        N.call("bbg_mlp_set_params", self.h, _fptr(a))

    def mlp_set_trained(self, substeps):
        N.call("bbg_mlp_set_trained", self.h, int(substeps))

    def mlp_status(self):
        t, s, l = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        N.call("bbg_mlp_status", self.h, ctypes.byref(t), ctypes.byref(s), ctypes.byref(l))
        return {"trained_substeps": t.value, "adam_steps": s.value, "last_loss": l.value}

    def mlp_infer(self, features):
        f = np.ascontiguousarray(features, dtype=np.float32).reshape(-1, 4)
        out = np.zeros(len(f), np.float32)
        N.call("bbg_mlp_infer", self.h, _fptr(f), len(f), _fptr(out))
        return out

    def mlp_train_batch(self, features, targets):
        f = np.ascontiguousarray(features, dtype=np.float32).reshape(-1, 4)
        t = np.ascontiguousarray(targets, dtype=np.float32).reshape(len(f))
        N.call("bbg_mlp_train_batch", self.h, _fptr(f), _fptr(t), len(f))

    def mlp_features(self):
        out = np.zeros((self.n, 4), np.float32)
        N.call("bbg_mlp_get_features", self.h, _fptr(out))
        return out

    def neighbor_counts(self):
        out = np.zeros(self.n, np.int32)
        N.call("bbg_neighbor_counts", self.h, out.ctypes.data_as(N._IP))
        return out

    def neighbor_lists(self, max_per_particle=64):
        """Neighbour sets of the last density pass: (counts, ids) with counts[i] the members
        of i other than itself and ids[i, :counts[i]] their caller ids (visit order, -1 past
        the end; rows truncated at max_per_particle)."""
        counts = np.zeros(self.n, np.int32)
        ids = np.zeros((self.n, max_per_particle), np.int32)
        N.call("bbg_neighbor_lists", self.h, int(max_per_particle), counts.ctypes.data_as(N._IP),
               ids.ctypes.data_as(N._IP) if max_per_particle else None)
        return counts, ids


class BatchSolver(Solver):
    """Independent scenes advanced together (bbg_batch_create): `scene` holds the shared
    parameters (spacing, density, corrector controls, pressure start, MLP settings),
    `boxes` each scene's container (box_min, box_max) and `positions` its particles."""

    def __init__(self, scene, boxes, positions, velocities=None, device=0, setup=True):
        self.scene = dict(scene)
        self.desc = desc_from_scene(dict(scene, domain_min=(0.0, 0.0, 0.0), domain_max=(1.0, 1.0, 1.0)),
                                    device)
        if len(boxes) != len(positions) or not boxes:
            raise ValueError("one container per scene")
        arr = (N.SceneDesc * len(boxes))()
        for i, ((lo, hi), p) in enumerate(zip(boxes, positions)):
            arr[i].count = len(p)
            for k in range(3):
                arr[i].box_min[k] = float(lo[k])
                arr[i].box_max[k] = float(hi[k])
        h = ctypes.c_void_p()
        N.call("bbg_batch_create", ctypes.byref(self.desc), arr, len(boxes), ctypes.byref(h))
        self.h = h
        self.counts = [len(p) for p in positions]
        self.n = 0
        if scene.get("pressure_init") == "learned" and scene.get("mlp"):
            self.mlp_configure(**scene["mlp"])
        self.upload_scenes(positions, velocities)
        if setup:
            self.setup()

    @property
    def scene_count(self):
        return len(self.counts)

    def layout(self):
        out = np.zeros((self.scene_count, 3))
        N.call("bbg_batch_layout", self.h, out.ctypes.data_as(N._DP))
        return out

    def upload_scenes(self, positions, velocities=None):
        p = np.ascontiguousarray(np.concatenate(positions), dtype=np.float32).reshape(-1, 3)
        v = None
        if velocities is not None:
            v = np.ascontiguousarray(np.concatenate(velocities), dtype=np.float32).reshape(-1, 3)
        N.call("bbg_batch_upload", self.h, _fptr(p), _fptr(v) if v is not None else None)
        self.n = int(p.shape[0])

    def download_scenes(self):
        """Per-scene positions and velocities in scene coordinates."""
        p = np.zeros((self.n, 3), np.float32)
        v = np.zeros((self.n, 3), np.float32)
        N.call("bbg_batch_download", self.h, _fptr(p), _fptr(v))
        cuts = np.cumsum(self.counts)[:-1]
        return np.split(p, cuts), np.split(v, cuts)

    def scene_stats(self):
        it = np.zeros(self.scene_count, np.int32)
        err = np.zeros(self.scene_count)
        N.call("bbg_batch_scene_stats", self.h, it.ctypes.data_as(N._IP), err.ctypes.data_as(N._DP))
        return it, err


class PciSphSolver3(Solver):
    """Reference-named facade of PciSphSolver3 (src/core/pcisph_solver.h:56-83)."""

    def Setup(self):
        self.setup()

    def SetColliders(self, colliders):
        self.set_colliders(colliders)

    def Advance(self, dt):
        return self.advance(dt)

    def GetParticleCount(self):
        return self.n

    def ComputeDelta(self, dt):
        return self.compute_delta(dt)


class SphSolver3(PciSphSolver3):
    """Reference-named facade of SphSolver3 (src/core/sph_solver.h:76-96)."""


def format_g(value):
    """printf("%g") of a float32 value through the frame writer's formatter (host)."""
    out = ctypes.create_string_buffer(16)
    n = ctypes.c_int()
    N.call("bbg_format_g", float(value), out, ctypes.byref(n))
    return out.raw[:n.value].decode()


def frame_section(text, flags=0):
    """The first fluid section of a frame text (host only): (flags, count, data_begin,
    data_end) with the data lines at text[data_begin:data_end]."""
    fl, cnt = ctypes.c_int(int(flags)), ctypes.c_int()
    a, b = ctypes.c_size_t(), ctypes.c_size_t()
    N.call("bbg_frame_find_section", bytes(text), len(text), ctypes.byref(fl), ctypes.byref(cnt),
           ctypes.byref(a), ctypes.byref(b))
    return fl.value, cnt.value, a.value, b.value


def build_grid(domain_min, domain_max, spacing, scale):
    """UtilBuildGridForDomain in the reference's FP32 arithmetic (host only)."""
    a = (ctypes.c_double * 3)(*domain_min)
    b = (ctypes.c_double * 3)(*domain_max)
    dims = (ctypes.c_int * 3)()
    geo = (ctypes.c_double * 12)()
    N.call("bbg_build_grid", a, b, float(spacing), float(scale), dims, geo)
    return np.array(list(dims), np.int32), np.array(list(geo))


def compute_mass(lattice, density, spacing, kernel_radius):
    m = ctypes.c_double()
    N.call("bbg_compute_mass", int(lattice), float(density), float(spacing), float(kernel_radius),
           ctypes.byref(m))
    return m.value


def compute_delta_denom(spacing, kernel_radius):
    d = ctypes.c_double()
    N.call("bbg_compute_delta_denom", float(spacing), float(kernel_radius), ctypes.byref(d))
    return d.value
