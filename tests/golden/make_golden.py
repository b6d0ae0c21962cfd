"""Generate the golden fixtures in this directory from the reference itself.

Runs only where the reference checkout exists: oracle/ref/build_ref.py compiles the
reference's own SPH/PCISPH CPU path host-only, and oracle/refsim.py drives its classes
(single thread).  For two small seeded scenes and both builds (FP32 = `typedef float
Float`, FP64 = as shipped) it stores the inputs and the reference's outputs:

  pcisph_<v>.npz  1,440-particle PCISPH dam break (box + sphere): setup scalars and grid,
                  the cell chains after Setup and after 3 as-shipped substeps, bucket
                  counts, every particle field after those substeps, the fields after a
                  3-iteration corrector built from the reference's own sub-passes, and
                  positions after Advance(2e-3) with its CFL substep loop.
  sph_<v>.npz     800-particle SPH dam break: fields after 3 as-shipped substeps
                  (ComputePressureForceCPU integrating in place, single thread).
  frame_f32.npz   the particle frames SerializerSaveSphDataSet3 (third/serializer.cpp)
                  appends for the FP32 PCISPH state after those 3 substeps, with the
                  position/velocity/density/mass flags and with position only, beside the
                  state they print; what SerializerLoadParticles3 reads back from the first
                  frame; and a hand-written frame of awkward lines (comments, blank lines,
                  CR and CRLF ends, tabs, malformed and out-of-range numbers) with what the
                  reference reads from it.

  continuous_f32.npz  ContinuousParticleSetBuilder3 on the 1,440-particle scene: MapGrid
                  after Setup, positions moved by hand, then two MapGridEmit calls; the
                  particle arrays after each, for a capacity that holds them and one that
                  stops the first call (CONTINUOUS_CASES).
  sdf_f32.npz     a field-only collider (MakeSDFShape of the scene's sphere, core/shape.h):
                  its grid, FieldGrid3f::Sample / Gradient, Shape::ClosestPoint and IsInside
                  at probe points, and TimeIntegrationCPU's collision response of 4,000
                  particles driven into the walls and the field.
  mesh_f32.npz    GenerateShapeSDF of two triangle meshes (MakeMesh, shapes/bvh.cpp): a rotated
                  icosphere and a rotated torus (rays cross it up to four times), their
                  vertices and triangles beside the reference's grids and node values.
  lnm_f32.npz     LNMBoundary (boundaries/lnm.h, fast variant) levels of the 1,440-particle
                  scene after 3 as-shipped substeps and a fresh grid distribution, for
                  h = 0.01, 0.02, 0.04 and unbounded.
  boundary_f32.npz  the other boundary classifications of boundaries/lnm.h, xiaowei.h and
                  dilts.h (LNMBoundarySingle, LNMBoundaryExtended, LNMBoundary with the Xiaowei
                  and Dilts L2 filters, XiaoweiBoundary, DiltsSpokeBoundary) of a jittered BCC
                  sphere the reference's emitter made (srand(7)), with the densities the
                  reference computed; and DiltsSpokeTakeUniformPoint's points for r = 1.
  surface_f32.npz the surface app's particle field (ParticlesToSDF_Surface, Zhu-Bridson and
                  SPH, by spacing and by resolution) of the same sphere, the densities and
                  domain it used (its own pieces, checked equal to the app function called
                  directly), and the reference's MarchingCubes of the by-spacing fields.
  mc_f32.npz      MarchingCubes (reconstruction/marching_cubes.cpp) of two fields on a 21x22x23
                  grid: two overlapping spheres' distance (iso 0) and a random field (every
                  cube configuration): the reference's points, normals and triangles.
  emit_f32.npz    particles VolumeParticleEmitter3 (core/emitter.cpp) emitted after
                  srand(seed) for boxes and spheres, with and without jitter, explicit
                  bounds, a reversed box and a binding max_particles (EMIT_CASES).

    python tests/golden/make_golden.py           # every fixture
    python tests/golden/make_golden.py frames    # frame_f32.npz only
    python tests/golden/make_golden.py emit      # emit_f32.npz only
    python tests/golden/make_golden.py continuous    # continuous_f32.npz only
    python tests/golden/make_golden.py sdf       # sdf_f32.npz only
    python tests/golden/make_golden.py mesh      # mesh_f32.npz only
    python tests/golden/make_golden.py lnm       # lnm_f32.npz only
    python tests/golden/make_golden.py mc        # mc_f32.npz only
    python tests/golden/make_golden.py boundary  # boundary_f32.npz only
    python tests/golden/make_golden.py surface   # surface_f32.npz only
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from bubbles_gb300 import scenes  # noqa: E402
from oracle import oracle as O  # noqa: E402
from oracle import refsim as R  # noqa: E402

FIELDS = {"pos": O.POSITION, "vel": O.VELOCITY, "force": O.FORCE, "density": O.DENSITY,
          "pressure": O.PRESSURE, "pred_density": O.PRED_DENSITY,
          "pressure_force": O.PRESSURE_FORCE, "pred_pos": O.PRED_POSITION}


def pcisph_scene():
    return scenes.small_pcisph(seed=0)


def sph_scene():
    sc = scenes.base_scene("sph", 0.02, (0.6, 0.5, 0.6))
    sc["dt"] = 1e-4
    return sc, scenes.dam_block(sc, (10, 8, 10), seed=1)


def clean(scene):
    return json.loads(json.dumps(scene, default=lambda o: list(o) if hasattr(o, "__iter__") else float(o)))


def make(variant):
    out = {}
    sc, pos = pcisph_scene()
    r = R.RefSim(sc, pos, variant=variant)
    out["scene"] = np.array(json.dumps(clean(sc)))
    out["pos0"] = pos
    s = r.scalars_dict()
    out["scalars"] = np.array([s[k] for k in ("mass", "kernel_radius", "delta_denom",
                                              "mass_over_density_sq")])
    dims, geo = r.grid()
    out["grid_dims"], out["grid_geo"] = dims, geo
    out["setup_cell_of"], out["setup_counts"], out["setup_chains"] = r.cells()
    for _ in range(3):
        r.advance_time_step(sc["dt"])
    out["step3_cell_of"], out["step3_counts"], out["step3_chains"] = r.cells()
    out["step3_bucket_counts"], _ = r.buckets()
    for name, f in FIELDS.items():
        out["step3_" + name] = r.get(f)
    # 3-iteration corrector from the reference's sub-passes, after a fresh grid update
    r.update_grid_distribution()
    r.reset_higher_level()
    r.compute_particle_interaction()
    r.compute_density(1)
    r.compute_non_pressure_force()
    delta = r.compute_delta(sc["dt"])
    out["corr_delta"] = np.array(delta)
    for k in range(3):
        r.predict_velocity_and_position(sc["dt"], int(k == 0))
        r.predict_pressure(delta)
        r.predict_pressure_force()
    for name in ("pred_density", "pressure", "pressure_force", "pred_pos"):
        out["corr_" + name] = r.get(FIELDS[name])
    r.accumulate_and_integrate(sc["dt"])
    out["corr_pos"] = r.get(O.POSITION)
    out["corr_vel"] = r.get(O.VELOCITY)
    r.advance(2e-3)
    out["advance_pos"] = r.get(O.POSITION)
    np.savez_compressed(os.path.join(HERE, "pcisph_%s.npz" % variant), **out)

    sc2, pos2 = sph_scene()
    r2 = R.RefSim(sc2, pos2, variant=variant)
    o2 = {"scene": np.array(json.dumps(clean(sc2))), "pos0": pos2}
    for _ in range(3):
        r2.advance_time_step(sc2["dt"])
    for name in ("pos", "vel", "force", "density", "pressure"):
        o2["step3_" + name] = r2.get(FIELDS[name])
    np.savez_compressed(os.path.join(HERE, "sph_%s.npz" % variant), **o2)


# a frame section written by hand: the reader's corner cases (the reference reads it, the
# stored arrays are its result)
AWKWARD = (b"# a comment before the section\n"
           b"FluidBegin\n\t\"Type\" particles\n\t\"Count\" 10\n\t\"Format\" pv\n\t\"Spacing\" 0.02\n"
           b"\tDataBegin\n"
           b"\t\t0.1 0.2 0.3 1 2 3\n"
           b"\t\t-0.5 +0.25 1e-3 -1.5e+2 2.5E-1 0\n"
           b"\t\t7 8 9 0.000001 123456789 -0\r\n"
           b"\n"
           b"   # comment line inside data DataEnd\n"
           b"\t\t1.23456789012345 0.333333333333333333 1e10 1e-10 -7.25e+03 3.4028235e38\n"
           b"\t\t.5 nan -inf 1e+ 1.5e 12abc\n"
           b"  \t 5\t6\t7 8 9 10\n"
           b"\t\t1e-45 1e-46 2e38 4e38 1.17549435e-38 -3.14159265358979\r\t\t42\n"
           b"\t\t1.0e400 1e-400 00012.50000 -.25 +-1 0x10\n"
           b"\t\t0e500 1.e5 5e 7e- 0.1234567891234 99999999999999999999999\n"
           b"\tDataEnd\nFluidEnd\n")

FRAME_FLAGS = {"pvdm": 0x01 | 0x02 | 0x04 | 0x20, "p": 0x01}   # SERIALIZER_* (third/serializer.h)


def make_frames():
    sc, pos = pcisph_scene()
    r = R.RefSim(sc, pos, variant="f32")
    for _ in range(3):
        r.advance_time_step(sc["dt"])
    out = {"scene": np.array(json.dumps(clean(sc))), "pos0": pos,
           "mass": np.array(r.scalars_dict()["mass"])}
    for name in ("pos", "vel", "density"):
        out["step3_" + name] = r.get(FIELDS[name])
    for name, flags in FRAME_FLAGS.items():
        out["frame_" + name] = np.frombuffer(r.frame(flags), dtype=np.uint8)
    fl, p, v, d, _ = R.load_frame(r.frame(FRAME_FLAGS["pvdm"]), 0)
    out["load_pvdm_flags"], out["load_pvdm_pos"], out["load_pvdm_vel"], out["load_pvdm_density"] = \
        np.array(fl), p, v, d
    out["awkward_frame"] = np.frombuffer(AWKWARD, dtype=np.uint8)
    fl, p, v, d, _ = R.load_frame(AWKWARD, 0)
    out["awkward_flags"], out["awkward_pos"], out["awkward_vel"] = np.array(fl), p, v
    np.savez_compressed(os.path.join(HERE, "frame_f32.npz"), **out)


# emitter cases: shape, spacing, jitter, initial velocity, max particles, bounds, srand seed
EMIT_CASES = [
    ({"type": "sphere", "radius": 0.1, "center": (0.01, 0.02, 0.03)}, 0.02, 0.0, (0.0, 0.0, 0.0), None, None, 1),
    ({"type": "box", "size": (0.2, 0.1, 0.3), "center": (0.0, 0.0, 0.0)}, 0.02, 0.5, (1.0, 0.0, -0.5), None, None,
     7),
    ({"type": "sphere", "radius": 0.15, "center": (0.5, 0.4, 0.3)}, 0.013, 1.0, (0.0, 0.0, 0.0), None, None, 11),
    ({"type": "box", "size": (0.4, 0.2, 0.3), "center": (0.1, 0.2, -0.3), "reverse": True}, 0.02, 0.3,
     (0.0, 0.0, 0.0), None, ((-0.2, 0.0, -0.5), (0.3, 0.35, -0.1)), 3),
    ({"type": "box", "size": (0.3, 0.3, 0.3), "center": (0.0, 0.0, 0.0)}, 0.015, 0.2, (0.0, 0.0, 0.0), 1000, None,
     5),
]


def make_emit():
    out = {"cases": np.array(json.dumps(EMIT_CASES))}
    for i, (shape, sp, jit, vel, mx, bounds, seed) in enumerate(EMIT_CASES):
        p, v = R.emit_volume(shape, sp, jitter=jit, velocity=vel, seed=seed, bounds=bounds,
                             max_particles=mx if mx is not None else 2**31 - 1)
        out["pos_%d" % i], out["vel_%d" % i] = p, v
    np.savez_compressed(os.path.join(HERE, "emit_f32.npz"), **out)


def sdf_collision_inputs(sc, rng):
    """Positions and velocities driving particles into the container and the sphere."""
    lo, hi = np.array(sc["domain_min"]), np.array(sc["domain_max"])
    p = rng.uniform(lo - 0.01, hi + 0.01, size=(4000, 3))
    sph = sc["colliders"][1]
    p[:1500] = np.array(sph["center"]) + rng.normal(size=(1500, 3)) * sph["radius"] * 0.7
    v = rng.normal(size=p.shape) * 2.0
    return p.astype(np.float32), v.astype(np.float32)


def make_sdf():
    import ctypes
    sc, _ = pcisph_scene()
    sph = sc["colliders"][1]
    center = np.array(sph["center"], np.float64)
    rng = np.random.default_rng(21)
    p, v = sdf_collision_inputs(sc, rng)
    r = R.RefSim(sc, p, v)
    r.make_sdf_sphere_collider(1, center.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), sph["radius"], 0.01,
                               0.2)
    nodes, org, sp, vals = r.collider_sdf(1)
    out = {"scene": np.array(json.dumps(clean(sc))), "nodes": nodes, "origin": org, "spacing": sp,
           "values": vals, "pos_in": p, "vel_in": v}
    pts = (center + rng.normal(size=(800, 3)) * sph["radius"] * 0.9).astype(np.float32)
    pts[:100] = (center + rng.uniform(-0.5, 0.5, size=(100, 3))).astype(np.float32)   # beyond the grid too
    out["probe_points"] = pts
    for k, a in r.sdf_probe(1, pts.astype(np.float64)).items():
        out["probe_" + k] = a
    r.set(O.FORCE, np.zeros_like(p, dtype=np.float64))
    r.time_integration(1e-3)
    out["pos_out"] = r.get(O.POSITION)
    out["vel_out"] = r.get(O.VELOCITY)
    np.savez_compressed(os.path.join(HERE, "sdf_f32.npz"), **out)


def rotation(ax, ay, az):
    rx = np.array([[1, 0, 0], [0, np.cos(ax), -np.sin(ax)], [0, np.sin(ax), np.cos(ax)]])
    ry = np.array([[np.cos(ay), 0, np.sin(ay)], [0, 1, 0], [-np.sin(ay), 0, np.cos(ay)]])
    rz = np.array([[np.cos(az), -np.sin(az), 0], [np.sin(az), np.cos(az), 0], [0, 0, 1]])
    return rz @ ry @ rx


def icosphere(radius=0.2, center=(0.03, -0.02, 0.01), level=2, rot=(0.3, 0.5, 0.7)):
    """A subdivided icosahedron on a sphere, rotated off the axes (float32 vertices)."""
    t = (1 + 5 ** 0.5) / 2
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v = [np.array(x, float) / np.linalg.norm(x) for x in v]
    for _ in range(level):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = v[a] + v[b]
                v.append(m / np.linalg.norm(m))
                cache[key] = len(v) - 1
            return cache[key]
        nf = []
        for a, b, c in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf
    verts = np.array(v) @ rotation(*rot).T * radius + np.array(center)
    return verts.astype(np.float32).astype(np.float64), np.array(f, np.int32)


def torus(big=0.18, small=0.06, nu=24, nv=12, center=(-0.01, 0.02, 0.015), rot=(0.9, 0.2, 0.4)):
    """A rotated torus of nu x nv quads split into triangles (float32 vertices)."""
    verts, tris = [], []
    for i in range(nu):
        for j in range(nv):
            u, w = 2 * np.pi * i / nu, 2 * np.pi * j / nv
            verts.append(((big + small * np.cos(w)) * np.cos(u), (big + small * np.cos(w)) * np.sin(u),
                          small * np.sin(w)))
    for i in range(nu):
        for j in range(nv):
            a, b = i * nv + j, ((i + 1) % nu) * nv + j
            c, d = ((i + 1) % nu) * nv + (j + 1) % nv, i * nv + (j + 1) % nv
            tris += [(a, b, c), (a, c, d)]
    verts = np.array(verts) @ rotation(*rot).T + np.array(center)
    return verts.astype(np.float32).astype(np.float64), np.array(tris, np.int32)


def soup(count=300, seed=5):
    """Triangles of random size, position and orientation in index order with no spatial
    coherence (overlapping, not closed): the worst case for skipping tiles of triangles."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-0.2, 0.2, (count, 1, 3))
    v = (c + rng.normal(0.0, 0.05, (count, 3, 3))).astype(np.float32).reshape(-1, 3)
    return v, np.arange(3 * count, dtype=np.int32).reshape(-1, 3)


MESH_CASES = {"icosphere": (icosphere, 0.02, 0.1), "torus": (torus, 0.015, 0.15), "soup": (soup, 0.02, 0.1)}


def make_mesh():
    out = {}
    for name, (make, dx, margin) in MESH_CASES.items():
        v, t = make()
        nodes, org, sp, vals = R.mesh_sdf(v, t, dx, margin)
        out.update({name + "_vertices": v, name + "_triangles": t, name + "_dx": np.array(dx),
                    name + "_margin": np.array(margin), name + "_nodes": nodes, name + "_origin": org,
                    name + "_spacing": sp, name + "_values": vals})
    np.savez_compressed(os.path.join(HERE, "mesh_f32.npz"), **out)


def mc_fields():
    """The marching-cubes fixture's grid and its two fields (float32 node values)."""
    nodes = np.array([21, 22, 23], np.int32)
    org = np.array([-0.5, -0.52, -0.55])
    sp = np.array([0.05, 0.05, 0.05])
    i, j, k = np.meshgrid(np.arange(nodes[0]), np.arange(nodes[1]), np.arange(nodes[2]), indexing="ij")
    idx = np.stack([i.ravel(order="F"), j.ravel(order="F"), k.ravel(order="F")], axis=1)
    pos = org.astype(np.float32) + sp.astype(np.float32) * idx.astype(np.float32)
    blobs = np.minimum(np.linalg.norm(pos - np.array([0.03, 0.01, -0.02]), axis=1) - 0.3,
                       np.linalg.norm(pos - np.array([0.25, 0.2, 0.1]), axis=1) - 0.15).astype(np.float32)
    noise = np.random.default_rng(3).normal(size=len(pos)).astype(np.float32)
    return nodes, org, sp, {"blobs": blobs, "noise": noise}


def make_mc():
    nodes, org, sp, fields = mc_fields()
    out = {"nodes": nodes, "origin": org, "spacing": sp}
    for name, vals in fields.items():
        p, n, t = R.marching_cubes(nodes, org, sp, vals, 0.0)
        out.update({name + "_values": vals, name + "_points": p, name + "_normals": n, name + "_triangles": t})
    np.savez_compressed(os.path.join(HERE, "mc_f32.npz"), **out)


LNM_CASES = [(0.01, 0), (0.02, 0), (0.04, 0), (0.02, 1)]


def make_lnm():
    sc, p0 = pcisph_scene()
    r = R.RefSim(sc, p0)
    for _ in range(3):
        r.advance_time_step(sc["dt"])
    r.update_grid_distribution()
    out = {"scene": np.array(json.dumps(clean(sc))), "pos": r.get(O.POSITION),
           "cases": np.array(json.dumps(LNM_CASES))}
    for i, (h, unbounded) in enumerate(LNM_CASES):
        out["levels_%d" % i] = r.lnm(h, unbounded)
    np.savez_compressed(os.path.join(HERE, "lnm_f32.npz"), **out)


# boundary fixture: a jittered BCC sphere emitted by the reference in the small container
BOUNDARY_SPHERE = {"type": "sphere", "center": (0.0, -0.03, 0.0), "radius": 0.2}
BOUNDARY_CASES = {
    "single": [(0.02, 0), (0.04, 0), (0.02, 1)],
    "extended": [(0.02, 5, 0), (0.02, 2, 0), (0.02, -1, 0), (0.04, 5, 1)],
    "geometric": [(0.02, 1, 0), (0.04, 1, 0), (0.02, 2, 0)],
    "xiaowei": [0.02, 0.01],
}


def boundary_scene():
    sc = scenes.base_scene("pcisph", 0.02, (0.6, 0.5, 0.6))
    sc["dt"] = 4e-4
    pos, _ = R.emit_volume(BOUNDARY_SPHERE, 0.02, jitter=0.2, seed=7)
    return sc, pos


def make_boundary():
    sc, pos = boundary_scene()
    r = R.RefSim(sc, pos)
    r.update_grid_distribution()
    r.compute_density(0)
    out = {"scene": np.array(json.dumps(clean(sc))), "pos": r.get(O.POSITION), "density": r.get(O.DENSITY),
           "cases": np.array(json.dumps(BOUNDARY_CASES))}
    for i, (h, ub) in enumerate(BOUNDARY_CASES["single"]):
        out["single_%d" % i] = r.lnm_single(h, ub)
    for i, (h, ml, ub) in enumerate(BOUNDARY_CASES["extended"]):
        out["extended_%d" % i] = r.lnm_extended(h, ml, ub)
    for i, (h, alg, ub) in enumerate(BOUNDARY_CASES["geometric"]):
        lv, q, a = r.lnm_geometric(h, alg, ub)
        out["geometric_%d" % i], out["geometric_stats_%d" % i] = lv, np.array([q, a], np.int32)
    for i, h in enumerate(BOUNDARY_CASES["xiaowei"]):
        out["xiaowei_%d" % i] = r.xiaowei(h)
    out["dilts"] = r.dilts()
    out["dilts_points"] = R.dilts_points()
    np.savez_compressed(os.path.join(HERE, "boundary_f32.npz"), **out)


# surface fixture: (method, resolution or None) of ParticlesToSDF_Surface on the boundary
# fixture's sphere, kernel radius 0.04, marching-cubes spacing 0.02
SURFACE_CASES = [(0, None), (1, None), (0, (40, 36, 44)), (1, (40, 36, 44))]


def make_surface():
    pos, _ = R.emit_volume(BOUNDARY_SPHERE, 0.02, jitter=0.2, seed=7)
    out = {"pos": pos, "cases": np.array(json.dumps(SURFACE_CASES))}
    for i, (method, res) in enumerate(SURFACE_CASES):
        r = R.surface_sdf(pos, 0.02, 0.04, 0.02, method, resolution=res)
        d = R.surface_sdf(pos, 0.02, 0.04, 0.02, method, resolution=res, direct=True)
        assert np.array_equal(r["values"].view(np.uint32), d["values"].view(np.uint32))
        for k in ("nodes", "origin", "spacing", "values"):
            out["%s_%d" % (k, i)] = r[k]
        out["domain"], out["density"] = r["domain"], r["density"]
        if res is None:
            p, n, t = R.marching_cubes(r["nodes"], r["origin"], (float(r["spacing"]),) * 3, r["values"], 0.0)
            out["mc_points_%d" % i], out["mc_normals_%d" % i], out["mc_triangles_%d" % i] = p, n, t
    np.savez_compressed(os.path.join(HERE, "surface_f32.npz"), **out)


# continuous emission cases: builder capacity, MapGridEmit distance, velocity
CONTINUOUS_CASES = [(5000, 0.01, (0.1, 0.0, 0.0)), (1800, 0.01, (0.0, -0.5, 0.0))]


def moved_positions(pos):
    """The hand-moved positions of the continuous-emission fixture."""
    rng = np.random.default_rng(1)
    return pos + np.array([0.012, 0.0, 0.009]) + rng.normal(0.0, 0.002, pos.shape)


def make_continuous():
    sc, p0 = pcisph_scene()
    p1 = moved_positions(p0)
    out = {"scene": np.array(json.dumps(clean(sc))), "pos0": p0, "pos1": p1,
           "cases": np.array(json.dumps(CONTINUOUS_CASES))}
    for i, (cap, d, vel) in enumerate(CONTINUOUS_CASES):
        r = R.RefSim(sc, p0, continuous=cap)
        r.map_grid()
        r.set(O.POSITION, p1)
        for k in range(2):
            r.map_grid_emit(d, vel)
            out["pos_%d_%d" % (i, k)] = r.get(O.POSITION)
            out["vel_%d_%d" % (i, k)] = r.get(O.VELOCITY)
    np.savez_compressed(os.path.join(HERE, "continuous_f32.npz"), **out)


if __name__ == "__main__":
    if not R.available():
        sys.exit("the reference checkout is not available here; fixtures unchanged")
    what = sys.argv[1:]
    if not what:
        for v in ("f32", "f64"):
            make(v)
    if not what or what == ["frames"]:
        make_frames()
    if not what or what == ["emit"]:
        make_emit()
    if not what or what == ["continuous"]:
        make_continuous()
    if not what or what == ["sdf"]:
        make_sdf()
    if not what or what == ["mesh"]:
        make_mesh()
    if not what or what == ["lnm"]:
        make_lnm()
    if not what or what == ["mc"]:
        make_mc()
    if not what or what == ["boundary"]:
        make_boundary()
    if not what or what == ["surface"]:
        make_surface()
    print("\n".join(sorted(f for f in os.listdir(HERE) if f.endswith(".npz"))))
