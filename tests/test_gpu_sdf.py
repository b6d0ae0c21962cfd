"""Colliders with signed-distance fields (FieldGrid3f; MakeSDFShape; GenerateShapeSDF).

Pinned against the reference (tests/golden/sdf_f32.npz): a field-only collider built by
MakeSDFShape from the scene's sphere, its FieldGrid3f::Sample / Gradient,
Shape::ClosestPoint (ClosestPointBySDF) and IsInside at probe points, and the collision
response of TimeIntegrationCPU for particles driven into the walls and the field; the
device must reproduce each bit for bit.  GenerateShapeSDF of analytic shapes is compared
with the oracle's ClosestDistance / IsInside at the same node positions.
"""
import json
import os

import numpy as np
import pytest

import bubbles_gb300 as bb
from bubbles_gb300 import scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sdf_f32.npz")


def golden():
    d = np.load(GOLDEN, allow_pickle=False)
    return {k: d[k] for k in d.files}, json.loads(str(d["scene"]))


def same_bits(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def field_scene(sc):
    """The golden scene with its sphere replaced by a field-only collider."""
    cols = [sc["colliders"][0], {"type": "sdf"}]
    return dict(sc, colliders=cols)


def attach(s, g):
    s.set_sdf(1, g["nodes"], g["origin"], g["spacing"], g["values"])


def test_field_queries_match_reference(gpu):
    g, sc = golden()
    with bb.Solver(field_scene(sc), pos=g["pos_in"]) as s:
        attach(s, g)
        nodes, org, sp, vals = s.get_sdf(1)
        assert np.array_equal(nodes, g["nodes"]) and same_bits(vals, g["values"])
        q = s.collider_query(1, g["probe_points"])
        for k in ("sample", "gradient", "point", "normal", "distance"):
            assert same_bits(q[k], g["probe_" + k]), k
        assert np.array_equal(q["inside"], g["probe_inside"])


def test_field_collision_response_matches_reference(gpu):
    g, sc = golden()
    with bb.Solver(field_scene(sc), pos=g["pos_in"], vel=g["vel_in"]) as s:
        attach(s, g)
        s.update_grid_distribution()
        s.set(bb.FIELD_FORCE, np.zeros_like(g["pos_in"]))
        s.time_integration(1e-3)
        p, v = s.download()
    assert same_bits(p, g["pos_out"]) and same_bits(v, g["vel_out"])


def test_field_obstacle_in_a_dam_break(gpu, small):
    """A field-only sphere obstacle in the running scene: particles flow around it."""
    g, _ = golden()
    sc, pos = small
    with bb.Solver(field_scene(sc), pos=pos) as s:
        attach(s, g)
        for _ in range(40):
            st = s.advance_time_step(sc["dt"], stats=True)
        p, _ = s.download()
        assert st["out_of_grid"] == 0 and np.all(np.isfinite(p))
        q = s.collider_query(1, p)
        assert np.all(q["sample"] > -0.5 * sc["colliders"][1]["radius"])
    with pytest.raises(bb.BbgError):   # a field-only collider needs its field
        with bb.Solver(field_scene(sc), pos=pos) as t:
            t.advance_time_step(sc["dt"])


@pytest.mark.parametrize("which", [0, 1])
def test_generate_sdf_of_analytic_shapes(gpu, small, which):
    """GenerateShapeSDF on the device: grid sized as the reference sizes it, nodes signed
    max(|ClosestDistance|, 1e-5) with the oracle's ClosestDistance / IsInside."""
    sc, pos = small
    shape = sc["colliders"][which]
    with bb.Solver(sc, pos=pos) as s:
        s.generate_sdf(which, dx=0.02, margin=0.1)
        nodes, org, sp, vals = s.get_sdf(which)
        # sizing in float32, as the reference computes it
        f = np.float32
        if shape["type"] == "box":
            h = np.array([f(f(x) / 2.0) for x in shape["size"]], f)
        else:
            h = np.full(3, f(shape["radius"]), f)
        t = np.array(shape["center"], f)
        lo, hi = -h + t, h + t
        scale = hi - lo
        lo, hi = lo - scale * f(0.1), hi + scale * f(0.1)
        w, hgt, dep = hi - lo
        res = int(np.ceil(w / f(0.02)))
        assert nodes[0] == res + 1
        assert nodes[1] == int(np.ceil(f(f(res) * hgt) / w)) + 1 and nodes[2] == int(np.ceil(f(f(res) * dep) / w)) + 1
        assert np.allclose(org, lo, rtol=0, atol=0) and sp[0] == f(w / f(res))
        i, j, k = np.meshgrid(np.arange(nodes[0]), np.arange(nodes[1]), np.arange(nodes[2]), indexing="ij")
        idx = np.stack([i.ravel(order="F"), j.ravel(order="F"), k.ravel(order="F")], axis=1)
        pts = (org.astype(f) + sp.astype(f) * idx.astype(f)).astype(f)
        d, ins = O.shape_distance(shape, pts.astype(np.float64))
        psd = np.maximum(np.abs(d).astype(f), f(0.00001))
        want = np.where(ins != 0, -psd, psd).astype(f)
        assert same_bits(vals, want)
        # the attached field now resolves collisions (ClosestPointBySDF); the run stays sane
        for _ in range(5):
            s.advance_time_step(sc["dt"])
        p, _ = s.download()
        assert np.all(np.isfinite(p))


MESH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mesh_f32.npz")


@pytest.mark.parametrize("name", ["icosphere", "torus", "soup"])
def test_mesh_field_matches_reference(gpu, small, name):
    """GenerateShapeSDF of a triangle mesh: the grid and every node's distance equal the
    reference's; the inside sign too, except where two triangles tie for a ray's closest
    hit (none in these meshes)."""
    d = np.load(MESH, allow_pickle=False)
    sc, pos = small
    with bb.Solver(sc, pos=pos) as s:
        nodes, org, sp, vals, bounds, stuck = s.mesh_sdf(d[name + "_vertices"], d[name + "_triangles"],
                                                         float(d[name + "_dx"]), float(d[name + "_margin"]))
    assert stuck == 0
    assert np.array_equal(nodes, d[name + "_nodes"])
    assert same_bits(org, d[name + "_origin"]) and same_bits(sp, d[name + "_spacing"])
    want = d[name + "_values"]
    assert same_bits(np.abs(vals), np.abs(want))
    assert np.array_equal(vals < 0, want < 0)


def test_mesh_collider_in_a_dam_break(gpu, small):
    """A mesh obstacle (the icosphere moved into the fluid's path) collides through its
    field: after the run no particle is deep inside it."""
    d = np.load(MESH, allow_pickle=False)
    sc, pos = small
    v = d["icosphere_vertices"] * 0.5 + np.array([0.05, -0.12, 0.05])
    with bb.Solver(field_scene(sc), pos=pos) as s:
        s.set_mesh_collider(1, v, d["icosphere_triangles"], dx=0.01, margin=0.1)
        nodes, org, sp, vals = s.get_sdf(1)
        assert (vals < 0).sum() > 0
        for _ in range(40):
            st = s.advance_time_step(sc["dt"], stats=True)
        p, _ = s.download()
        assert st["out_of_grid"] == 0 and np.all(np.isfinite(p))
        q = s.collider_query(1, p)
        assert np.all(q["sample"] > -0.05)
