"""The allocation-free grid sort (bbg_grid_sort_noalloc) against the solver's grid.

bbg_grid_sort_noalloc exists for callers that cannot allocate device memory: it works
on device buffers the caller owns and keeps its scratch in a fixed array compiled into
the library.  The grid it returns must be the one a solver computes through
bbg_update_grid_distribution + bbg_dump_grid -- bit for bit, like every grid result
here -- on consecutive calls, since the calls share (and must clear) that scratch.

This file sorts last so that, when it fails, a run that stops at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

import bubbles_gb300 as bb
from bubbles_gb300 import _native as N
from bubbles_gb300 import scenes

pytestmark = pytest.mark.gpu


def noalloc_grid(torch, pos, scene):
    """Call the C entry point on torch-owned (caller-owned) device buffers; returns the
    cell of each particle, the sorted ids, the cell starts and the out-of-grid count."""
    n = len(pos)
    dims, _ = bb.build_grid(scene["domain_min"], scene["domain_max"], scene["spacing"],
                            scene["grid_spacing_scale"])
    cells = int(np.prod(dims))
    d_pos = torch.tensor(np.ascontiguousarray(pos, np.float32), device="cuda")
    d_cell = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    d_ids = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    d_start = torch.full((cells + 1,), -1, dtype=torch.int32, device="cuda")
    d_out = torch.full((1,), 12345, dtype=torch.int32, device="cuda")   # must be reset by the call
    lo = (ctypes.c_double * 3)(*scene["domain_min"])
    hi = (ctypes.c_double * 3)(*scene["domain_max"])
    stream = torch.cuda.current_stream()
    N.call("bbg_grid_sort_noalloc", ctypes.c_void_p(d_pos.data_ptr()), n, lo, hi,
           float(scene["spacing"]), float(scene["grid_spacing_scale"]),
           ctypes.c_void_p(d_cell.data_ptr()), ctypes.c_void_p(d_ids.data_ptr()),
           ctypes.c_void_p(d_start.data_ptr()), ctypes.c_void_p(d_out.data_ptr()),
           ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    as_u32 = lambda t: t.cpu().numpy().view(np.uint32)
    return as_u32(d_cell), as_u32(d_ids), as_u32(d_start), int(d_out.item())


def test_noalloc_grid_sort_matches_solver_grid(gpu):
    torch = pytest.importorskip("torch")
    sc, pos = scenes.pcisph_262k(seed=4)
    with bb.Solver(sc, pos=pos) as g:
        for call in range(2):   # two calls in a row: the second reuses the scratch
            p, _ = g.download()
            g.update_grid_distribution()
            cell_ref, counts_ref, ids_ref = g.dump_grid()
            cell, ids, start, outside = noalloc_grid(torch, p, sc)
            assert outside == 0, call
            assert np.array_equal(cell, cell_ref), call
            assert np.array_equal(ids, ids_ref), call
            assert start[0] == 0 and start[-1] == len(p)
            assert np.array_equal(np.diff(start.astype(np.int64)), counts_ref.astype(np.int64)), call
            for _ in range(15):   # move the particles before the second call
                g.advance_time_step(sc["dt"])


def test_noalloc_counts_particles_outside_the_grid(gpu):
    """Particles outside the domain are clamped into the edge cells, as in the solver's
    grid, and counted in the caller's counter."""
    torch = pytest.importorskip("torch")
    sc, pos = scenes.small_pcisph()
    p = np.array(pos, np.float32)
    p[7] = np.asarray(sc["domain_max"], np.float32) + np.float32(0.5)
    p[100, 0] = np.float32(sc["domain_min"][0]) - np.float32(0.25)
    with bb.Solver(sc, pos=p) as g:
        g.update_grid_distribution()
        cell_ref, _, ids_ref = g.dump_grid()
    cell, ids, _, outside = noalloc_grid(torch, p, sc)
    assert outside == 2
    assert np.array_equal(cell, cell_ref) and np.array_equal(ids, ids_ref)
    for _ in range(2):   # and the counter starts from zero on every call
        assert noalloc_grid(torch, pos, sc)[3] == 0


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    torch = pytest.importorskip("torch")
    sc, _ = scenes.pcisph_1m(positions=False)
    lo = (ctypes.c_double * 3)(*sc["domain_min"])
    hi = (ctypes.c_double * 3)(*sc["domain_max"])
    d = torch.zeros(16, dtype=torch.int32, device="cuda")
    ptr = ctypes.c_void_p(d.data_ptr())
    with pytest.raises(bb.BbgError) as e:   # more particles than the fixed scratch holds
        N.call("bbg_grid_sort_noalloc", ptr, 1048577, lo, hi, 0.008, 2.0, ptr, ptr,
               ptr, None, None)
    assert e.value.status == 4
    with pytest.raises(bb.BbgError) as e:   # a grid with more cells than the scratch holds
        N.call("bbg_grid_sort_noalloc", ptr, 4, lo, hi, 0.002, 2.0, ptr, ptr, ptr, None, None)
    assert e.value.status == 4
