"""Marching cubes on the device against the reference's MarchingCubes
(tests/golden/mc_f32.npz).

Points and normals are the reference's bit for bit (compared as sets keyed by position:
the device orders points by edge, the reference by first use).  Triangles are the
reference's: the same triangles with the same orientation, compared as a multiset of
vertex triples (each triple of points' bit patterns rotated to start at its smallest, so
the winding is kept), on the smooth field and on the random field (every cube
configuration, many ambiguous faces).  The smooth surface is also closed and faces outwards.
"""
import os

import numpy as np
import pytest

import bubbles_gb300 as bb

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mc_f32.npz")


def keyed(points, normals):
    order = np.lexsort((points[:, 2], points[:, 1], points[:, 0]))
    return points[order], normals[order]


def same_bits(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def triangle_keys(points, tris):
    """Each triangle as its three points' bit patterns, rotated to start at the smallest
    (orientation kept), sorted into a list."""
    bits = [tuple(r) for r in np.ascontiguousarray(points, np.float32).view(np.uint32)]
    out = []
    for a, b, c in tris:
        t = (bits[a], bits[b], bits[c])
        k = t.index(min(t))
        out.append(t[k:] + t[:k])
    out.sort()
    return out


@pytest.mark.parametrize("name", ["blobs", "noise"])
def test_triangles_match_reference(gpu, small, name):
    d = np.load(GOLDEN, allow_pickle=False)
    sc, pos = small
    with bb.Solver(sc, pos=pos) as s:
        p, _, t = s.marching_cubes(d["nodes"], d["origin"], d["spacing"], d[name + "_values"], 0.0)
    assert len(t) == len(d[name + "_triangles"])
    assert triangle_keys(p, t) == triangle_keys(d[name + "_points"], d[name + "_triangles"])


@pytest.mark.parametrize("name", ["blobs", "noise"])
def test_points_and_normals_match_reference(gpu, small, name):
    d = np.load(GOLDEN, allow_pickle=False)
    sc, pos = small
    with bb.Solver(sc, pos=pos) as s:
        p, n, t = s.marching_cubes(d["nodes"], d["origin"], d["spacing"], d[name + "_values"], 0.0)
    mp, mn = keyed(p, n)
    rp, rn = keyed(d[name + "_points"], d[name + "_normals"])
    assert same_bits(mp, rp) and same_bits(mn, rn)
    assert t.min() >= 0 and t.max() < len(p)


def test_smooth_surface_is_closed_and_outward(gpu, small):
    d = np.load(GOLDEN, allow_pickle=False)
    sc, pos = small
    with bb.Solver(sc, pos=pos) as s:
        p, n, t = s.marching_cubes(d["nodes"], d["origin"], d["spacing"], d["blobs_values"], 0.0)
        _, _, tr = s.marching_cubes(d["nodes"], d["origin"], d["spacing"], d["blobs_values"], 0.0,
                                    rotate_faces=True)
    assert len(t) == len(d["blobs_triangles"])
    # closed: every directed edge appears once and its reverse once
    e = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
    fwd = set(map(tuple, e))
    assert len(fwd) == len(e) and all((b, a) in fwd for a, b in fwd)
    # outward: the geometric normal agrees with the interpolated gradient normal
    a, b, c = p[t[:, 0]], p[t[:, 1]], p[t[:, 2]]
    geo = np.cross(b - a, c - a)
    assert np.mean(np.sum(geo * (n[t[:, 0]] + n[t[:, 1]] + n[t[:, 2]]), axis=1) > 0) > 0.99
    assert np.array_equal(tr, t[:, [0, 2, 1]])


def test_repeated_calls_reuse_the_solver_scratch(gpu, small):
    """Post-processing calls take their device buffers from the solver's scratch, which
    keeps its size between calls and grows when a call needs more: the same results on a
    solver that ran other, smaller calls before, in any order."""
    d = np.load(GOLDEN, allow_pickle=False)
    sc, pos = small
    args = {name: (d["nodes"], d["origin"], d["spacing"], d[name + "_values"], 0.0) for name in ("blobs", "noise")}
    with bb.Solver(sc, pos=pos) as fresh:
        want = {name: fresh.marching_cubes(*a) for name, a in args.items()}
    nx, ny, nz = (int(v) for v in d["nodes"])
    part = (nx // 2 + 1, ny // 2 + 1, nz // 2 + 1)   # a corner of the blobs field
    corner = d["blobs_values"].reshape(nz, ny, nx)[:part[2], :part[1], :part[0]].ravel()
    with bb.Solver(sc, pos=pos) as s:
        for name in ("noise", "blobs", "noise"):
            s.marching_cubes(part, d["origin"], d["spacing"], corner, 0.0)
            got = s.marching_cubes(*args[name])
            p, n, t = got
            wp, wn, wt = want[name]
            assert same_bits(p, wp) and same_bits(n, wn) and np.array_equal(t, wt)
