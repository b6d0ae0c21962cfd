"""The C++ side of the boundary without a GPU.

- bbg_bubbles.hpp (the reference's PciSphSolver3 / SphSolver3 API over the C ABI) compiles
  with -Wall -Werror, links with libbbg, and a program using it fails cleanly with
  BBG_ERR_NO_DEVICE where there is no GPU (tests/test_gpu_facade.py runs it on one).
- The reference-side binding (bubbles_gb300/bridge/pcisph_bbg.cpp) compiles against the
  reference's own headers and links with the reference's host build and libbbg: a program
  built from the reference's classes attaches libbbg (where the reference checkout and its
  host build exist; skipped elsewhere).
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from cpp_build import LIB_DIR, ROOT, compile_program, write_scene

REF_DIR = os.path.join(ROOT, "oracle", "ref")


def test_facade_compiles_links_and_reports_no_device(tmp_path):
    from bubbles_gb300 import build, scenes
    build.build()
    exe = compile_program("facade_advance.cpp", tmp_path / "facade_advance")
    sc, pos = scenes.small_pcisph()
    write_scene(tmp_path / "in.bin", sc, pos)
    p = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    from bubbles_gb300 import _native
    if _native.device_count() > 0:
        assert p.returncode == 0, p.stdout
    else:
        assert p.returncode == 6, p.stdout          # BBG_ERR_NO_DEVICE
        assert "bbg_create" in p.stdout


def test_reference_binding_builds_against_reference_headers(tmp_path):
    sys.path.insert(0, REF_DIR)
    try:
        import build_ref
    finally:
        sys.path.remove(REF_DIR)
    if not build_ref.available():
        pytest.skip("reference checkout not present")
    libs = build_ref.build()
    ref_lib = build_ref.lib_path("f64")
    if ref_lib not in libs or not os.path.exists(ref_lib):
        pytest.skip("reference host build unavailable")
    from bubbles_gb300 import build
    build.build()
    gen = os.path.join(build_ref.OUT, "gen_f64")
    flags = ["-I", gen, "-I", build_ref.SHIM] + sum([["-I", os.path.join(build_ref.SRC, d)] for d in build_ref.INC], [])
    exe = tmp_path / "bridge_main"
    cmd = (["g++", "-std=c++17", "-O1", "-w", "-pthread", "-I", os.path.join(ROOT, "include")] + flags +
           [os.path.join(ROOT, "tests", "cpp", "bridge_main.cpp"),
            os.path.join(ROOT, "bubbles_gb300", "bridge", "pcisph_bbg.cpp"),
            ref_lib, "-L", LIB_DIR, "-lbbg", "-Wl,-rpath," + LIB_DIR + ":" + os.path.dirname(ref_lib),
            "-o", str(exe)])
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert p.returncode == 0, p.stdout[-4000:]
    r = subprocess.run([str(exe)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:]
    from bubbles_gb300 import _native
    if _native.device_count() > 0:
        assert "advance 0" in r.stdout
    else:
        assert "attach 6" in r.stdout               # bbg_create: BBG_ERR_NO_DEVICE
