"""bbg_step_host: one substep with the state in host memory equals the separate calls it
stands for (upload, set the carried pressure, advance, download, get the pressure), bit for
bit, over several substeps of a warm-started corrector, with pageable host arrays and with
pinned ones (asynchronous copies, read back only after the step's synchronisation)."""
import numpy as np
import pytest

import bubbles_gb300 as bb

pytestmark = pytest.mark.gpu


def host_array(a, pinned):
    if not pinned:
        return a.copy()
    import torch
    t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True).numpy()
    t[...] = a
    return t


@pytest.mark.parametrize("pinned", [False, True])
def test_step_host_equals_the_separate_calls(gpu, small, pinned):
    sc, pos = small
    sc = dict(sc, pressure_init="previous", pcisph_mode="tolerance")
    p0 = np.ascontiguousarray(pos, np.float32)
    v0 = np.zeros_like(p0)
    pr0 = np.zeros(len(p0), np.float32)
    with bb.Solver(sc, pos=p0) as a, bb.Solver(sc, pos=p0) as b:
        pa, va, ra = p0.copy(), v0.copy(), pr0.copy()
        pb, vb, rb = host_array(p0, pinned), host_array(v0, pinned), host_array(pr0, pinned)
        for _ in range(4):
            a.upload(pa, va)
            a.set(bb.FIELD_PRESSURE, ra)
            a.advance_time_step(sc["dt"])
            pa, va = a.download()
            ra = a.get(bb.FIELD_PRESSURE)
            b.step_host(sc["dt"], pb, vb, rb, None, pb, vb, rb, None)
        assert np.array_equal(pa.view(np.uint32), pb.view(np.uint32))
        assert np.array_equal(va.view(np.uint32), vb.view(np.uint32))
        assert np.array_equal(np.asarray(ra, np.float32).view(np.uint32), rb.view(np.uint32))
        with pytest.raises(bb.BbgError):
            b.step_host(sc["dt"], pb, vb, None, rb, pb, vb, None, rb)   # no learned warm start
