"""The surface app's particle-to-field step (apps/surface.cpp: ParticlesToSDF_Surface with
ZhuBridsonSDF or SphSDF) on the sorted grid, and the whole app on the device (particles ->
field -> MarchingCubes).

The oracle's restatement (oracle/sph_oracle.c, orc_particle_sdf) is pinned against the field
the reference computed (tests/golden/surface_f32.npz, by spacing and by resolution, both
methods, with the densities it used); the device is compared with both bit for bit, and
the end-to-end mesh's points and normals with the reference's MarchingCubes of its field.
"""
import json
import os

import numpy as np
import pytest

import bubbles_gb300 as bb
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "surface_f32.npz")
KERNEL, MC_SPACING, SPACING = 0.04, 0.02, 0.02


def golden():
    d = np.load(GOLDEN, allow_pickle=False)
    return {k: d[k] for k in d.files}, json.loads(str(d["cases"]))


def same_bits(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def keyed(points, normals):
    order = np.lexsort((points[:, 2], points[:, 1], points[:, 0]))
    return points[order], normals[order]


def test_surface_domain_is_the_reference():
    g, _ = golden()
    sc = bb.surface_scene(g["pos"], SPACING)
    dims, geo = bb.build_grid(sc["domain_min"], sc["domain_max"], SPACING, 2.0)
    assert same_bits(geo[6:12], g["domain"])


def test_oracle_field_is_the_reference():
    g, cases = golden()
    o = O.OracleSim(bb.surface_scene(g["pos"], SPACING), g["pos"])
    o.update_grid_distribution()
    o.compute_density(0)
    assert same_bits(o.get(O.DENSITY), g["density"])
    for i, (method, res) in enumerate(cases):
        nodes, org, sp, vals = o.particle_sdf(method, KERNEL, MC_SPACING, res)
        assert np.array_equal(nodes, g["nodes_%d" % i]) and same_bits(org, g["origin_%d" % i])
        assert same_bits(sp, g["spacing_%d" % i]) and same_bits(vals, g["values_%d" % i]), (method, res)
    o.close()


@pytest.mark.gpu
def test_device_field_matches_reference(gpu):
    g, cases = golden()
    with bb.Solver(bb.surface_scene(g["pos"], SPACING), pos=g["pos"]) as s:
        s.update_grid_distribution()
        s.set(bb.FIELD_DENSITY, g["density"])
        for i, (method, res) in enumerate(cases):
            nodes, org, sp, vals = s.particle_sdf(method, KERNEL, MC_SPACING, res)
            assert np.array_equal(nodes, g["nodes_%d" % i]) and same_bits(org, g["origin_%d" % i])
            assert np.all(sp == g["spacing_%d" % i]) and same_bits(vals, g["values_%d" % i]), (method, res)
        with pytest.raises(bb.BbgError):
            s.particle_sdf(7, KERNEL, MC_SPACING)


@pytest.mark.gpu
def test_reconstruct_surface_end_to_end(gpu):
    """The app on the device: the Zhu-Bridson mesh's points and normals are the reference's
    (its MarchingCubes of its field); the SPH mesh, whose field depends on the device's own
    densities, agrees in shape."""
    g, _ = golden()
    p, n, t = bb.reconstruct_surface(g["pos"], SPACING, KERNEL, MC_SPACING, "zhu")
    mp, mn = keyed(p, n)
    rp, rn = keyed(g["mc_points_0"], g["mc_normals_0"])
    assert same_bits(mp, rp) and same_bits(mn, rn)
    assert len(t) == len(g["mc_triangles_0"])
    p, n, t = bb.reconstruct_surface(g["pos"], SPACING, KERNEL, MC_SPACING, "sph")
    assert abs(len(p) - len(g["mc_points_1"])) <= 2 and len(t) > 0


@pytest.mark.gpu
def test_field_full_size_against_oracle(gpu):
    """The 1,048,576-particle dam block: both methods' fields equal the oracle's on the same
    distribution and densities."""
    _, pos = bb.scenes.pcisph_1m()
    sp = 0.008
    sc = bb.surface_scene(pos, sp)
    o = O.OracleSim(sc, pos)
    o.update_grid_distribution()
    o.compute_density(0)
    rho = o.get(O.DENSITY)
    want = [o.particle_sdf(m, 2 * sp, sp) for m in (0, 1)]
    o.close()
    with bb.Solver(sc, pos=pos) as s:
        s.update_grid_distribution()
        s.set(bb.FIELD_DENSITY, rho)
        for m in (0, 1):
            nodes, org, spc, vals = s.particle_sdf(m, 2 * sp, sp)
            assert np.array_equal(nodes, want[m][0]) and same_bits(vals, want[m][3]), m
            assert (vals < 0).sum() > 0 and (vals > 0).sum() > 0
