"""FP64 mass / energy / momentum reductions of the particle state (bbg_energy), against the
same sums in numpy FP64 over the downloaded state."""
import numpy as np
import pytest

import bubbles_gb300 as bb

pytestmark = pytest.mark.gpu


def test_energy_matches_numpy(gpu, small):
    sc, pos = small
    with bb.Solver(sc, pos=pos) as s:
        for _ in range(5):
            s.advance_time_step(sc["dt"])
        p, v = s.download()
        e = s.energy()
        m = s.scalars()["mass"]
    p = p.astype(np.float64)
    v = v.astype(np.float64)
    g = np.array(sc["gravity"], np.float64)
    assert e["mass"] == pytest.approx(m * len(p), rel=1e-12)
    assert e["kinetic"] == pytest.approx(0.5 * m * np.sum(v * v), rel=1e-10)
    assert e["potential"] == pytest.approx(-m * np.sum(p @ g), rel=1e-10, abs=1e-12)
    assert np.allclose(e["momentum"], m * v.sum(axis=0), rtol=1e-10, atol=1e-12)
    assert e["kinetic"] > 0


def test_energy_is_repeatable(gpu, small):
    sc, pos = small
    with bb.Solver(sc, pos=pos) as s:
        s.advance_time_step(sc["dt"])
        a, b = s.energy(), s.energy()
    assert a["kinetic"] == b["kinetic"] and a["potential"] == b["potential"]


def test_nonfinite_state_is_counted(gpu, small):
    """Failure detection without a GPU fault: a NaN planted in the host input spreads
    through its neighbours and the step reports the non-finite particles; a healthy run
    reports none."""
    sc, pos = small
    with bb.Solver(sc, pos=pos) as s:
        st = s.advance_time_step(sc["dt"], stats=True)
        assert st["nonfinite"] == 0
    bad = np.array(pos, np.float32)
    bad[len(bad) // 2, 1] = np.nan
    with bb.Solver(sc, pos=bad) as s:
        st = s.advance_time_step(sc["dt"], stats=True)
        assert st["nonfinite"] >= 1
        p, _ = s.download()
        assert np.isnan(p).any(axis=1).sum() == st["nonfinite"]


def test_allocation_failures_are_reported(gpu, small):
    """Allocation failure without a GPU fault: an injected failure at each point of the
    solver's allocations (BBG_FAIL_ALLOC_AFTER, in a child process) and a request far past
    the device's memory both come back as BBG_ERR_OUT_OF_MEMORY, and the process goes on."""
    import os
    import subprocess
    import sys
    sc, pos = small
    code = ("import numpy as np, bubbles_gb300 as bb\n"
            "from bubbles_gb300 import scenes\n"
            "sc, pos = scenes.small_pcisph()\n"
            "try:\n"
            "    bb.Solver(sc, pos=pos).close()\n"
            "    print('created')\n"
            "except bb.BbgError as e:\n"
            "    print('status', e.status)\n")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for k in (0, 4, 17):
        env = dict(os.environ, BBG_FAIL_ALLOC_AFTER=str(k), PYTHONPATH=root)
        out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
        assert out.returncode == 0, out.stderr[-2000:]
        assert "status 3" in out.stdout, out.stdout
    with pytest.raises(bb.BbgError) as e:
        bb.Solver(sc, pos=pos, capacity=1 << 30)   # ~300 GB of particle state
    assert e.value.status == 3
    with bb.Solver(sc, pos=pos) as s:              # the device is still usable
        assert s.advance_time_step(sc["dt"], stats=True)["nonfinite"] == 0
