"""C-ABI checks that need no GPU: the library loads, exports every entry point the
header declares, validates arguments, refuses to run without a device, and its FP32
setup math (grid, mass, delta denominator) equals the FP32 oracle bit for bit."""
import ctypes
import os
import re

import numpy as np
import pytest

from bubbles_gb300 import _native as N
from bubbles_gb300 import scenes, solver
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for fname in os.listdir(os.path.join(ROOT, "include")):
        if not fname.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", fname)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(bbg_[a-z_0-9]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol(native):
    lib = native.load()
    names = declared_functions()
    assert len(names) >= 30
    for name in names:
        assert hasattr(lib, name), name


def test_version_and_status_strings(native):
    lib = native.load()
    assert b"sm_103a" in lib.bbg_version()
    assert lib.bbg_status_string(0) == b"ok"
    assert lib.bbg_status_string(6) == b"no CUDA device"


def test_desc_defaults_match_reference(native):
    # DefaultSphSolverData3, src/solvers/sph_solver3.cpp:124-151
    d = N.SolverDesc()
    N.call("bbg_solver_desc_default", ctypes.byref(d), N.SOLVER_PCISPH)
    assert (d.eos_exponent, d.negative_pressure_scale, d.viscosity) == (7.0, 0.0, 0.04)
    assert (d.pseudo_viscosity, d.sound_speed, d.drag_coefficient) == (10.0, 100.0, 0.0001)
    assert abs(d.gravity[1] + 9.8) < 1e-6 and d.time_step_limit_scale == 5.0
    assert d.max_iterations == 5 and d.max_density_error_ratio == 0.01
    with pytest.raises(N.BbgError) as e:
        N.call("bbg_solver_desc_default", ctypes.byref(d), 7)
    assert e.value.status == 1


def test_create_validates_arguments(native):
    d = N.SolverDesc()
    N.call("bbg_solver_desc_default", ctypes.byref(d), N.SOLVER_PCISPH)
    h = ctypes.c_void_p()
    with pytest.raises(N.BbgError) as e:   # empty domain
        N.call("bbg_create", ctypes.byref(d), 10, ctypes.byref(h))
    assert e.value.status == 1
    with pytest.raises(N.BbgError):
        N.call("bbg_create", ctypes.byref(d), 0, ctypes.byref(h))


def test_no_device_is_an_error_not_a_fallback(native):
    if native.device_count() > 0:
        pytest.skip("a GPU is visible")
    sc, _ = scenes.small_pcisph()
    d = solver.desc_from_scene(sc)
    h = ctypes.c_void_p()
    with pytest.raises(N.BbgError) as e:
        N.call("bbg_create", ctypes.byref(d), 100, ctypes.byref(h))
    assert e.value.status == 6


@pytest.mark.parametrize("name", sorted(scenes.CONFIGS))
def test_grid_geometry_matches_fp32_oracle(native, name):
    sc, _ = scenes.config(name, positions=False)
    d1, g1, _ = O.build_grid(sc["domain_min"], sc["domain_max"], sc["spacing"], 2.0)
    d2, g2 = solver.build_grid(sc["domain_min"], sc["domain_max"], sc["spacing"], 2.0)
    assert np.array_equal(d1, d2) and np.array_equal(g1, g2)


def test_grid_geometry_random_domains(native):
    rng = np.random.default_rng(11)
    for _ in range(200):
        lo = rng.uniform(-3, 0, 3)
        hi = lo + rng.uniform(0.1, 4, 3)
        sp = rng.uniform(0.003, 0.05)
        d1, g1, _ = O.build_grid(lo, hi, sp, 2.0)
        d2, g2 = solver.build_grid(lo, hi, sp, 2.0)
        assert np.array_equal(d1, d2) and np.array_equal(g1, g2)


@pytest.mark.parametrize("spacing", [0.005, 0.008, 0.01, 0.02, 0.1])
def test_mass_and_delta_denominator_match_fp32_oracle(native, spacing):
    kr = np.float32(2.0) * np.float32(spacing)
    assert solver.compute_mass(0, 1000.0, spacing, float(kr)) == O.compute_mass_bcc(1000.0, spacing, float(kr))
    assert solver.compute_delta_denom(spacing, float(kr)) == O.compute_delta_denom(spacing, float(kr))
    # cubic-lattice mass agrees with the FP64 scene value to FP32 rounding
    m = solver.compute_mass(1, 1000.0, spacing, float(kr))
    assert abs(m - scenes.cubic_mass(1000.0, spacing, 2 * spacing)) < 2e-6 * m
