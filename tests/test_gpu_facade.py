"""The reference's C++ solver API over libbbg on the GPU (include/bbg_bubbles.hpp).

A C++ program written the way a Bubbles program is (Initialize, Setup, SetColliders,
Advance) is compiled here against bbg_bubbles.hpp, run on the device, and compared with
the oracle's restatement of PciSphSolver3::Advance / SphSolver3::Advance
(src/solvers/pcisph_solver3.cpp:67-89, sph_solver3.cpp:69-93) on the same scene: the same
number of CFL substeps, positions within 1e-3 x spacing after the Advance (FP32 sums in
another order, over several substeps, as in tests/test_gpu_parity.py).
"""
import subprocess

import numpy as np
import pytest

from bubbles_gb300 import scenes
from cpp_build import compile_program, read_result, write_scene
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def facade(gpu, tmp_path_factory):
    return compile_program("facade_advance.cpp", tmp_path_factory.mktemp("facade") / "facade_advance")


def run(exe, tmp_path, sc, pos, kind, mode, count, dt):
    write_scene(tmp_path / "in.bin", sc, pos, kind=kind, mode=mode, count=count, dt=dt)
    p = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300)
    assert p.returncode == 0, p.stdout
    print(p.stdout.strip())
    return read_result(tmp_path / "out.bin", len(pos))


@pytest.mark.parametrize("mode", [O.PCISPH_AS_SHIPPED, O.PCISPH_TOLERANCE])
def test_pcisph_advance_through_cpp_facade(facade, tmp_path, mode):
    sc, pos = scenes.small_pcisph()
    x, v, substeps = run(facade, tmp_path, sc, pos, 0, mode, 1, 2e-3)
    o = O.OracleSim(sc, pos, variant="f32")
    steps = o.advance_pcisph(2e-3, 0.01, 5 if mode == O.PCISPH_AS_SHIPPED else 20, mode)[0]
    assert substeps == steps
    assert np.max(np.abs(x - o.get(O.POSITION))) <= 1e-3 * sc["spacing"]
    o.close()


def test_sph_advance_through_cpp_facade(facade, tmp_path):
    sc, pos = scenes.sph_16k(seed=3)
    x, v, substeps = run(facade, tmp_path, sc, pos, 1, 0, 2, sc["dt"])
    o = O.OracleSim(sc, pos, variant="f32")
    o.advance_sph(sc["dt"])
    steps = o.advance_sph(sc["dt"])
    assert substeps == steps
    assert np.max(np.abs(x - o.get(O.POSITION))) <= 1e-3 * sc["spacing"]
    o.close()
