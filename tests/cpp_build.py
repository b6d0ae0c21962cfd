"""Build helpers for the C++ programs under tests/cpp (test infrastructure): they are
compiled with g++ against include/ and linked with the in-tree libbbg."""
import os
import struct
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(ROOT, "bubbles_gb300", "_lib")


def compile_program(source, out, extra=()):
    """g++ -std=c++17 of tests/cpp/<source> into `out`, linked with libbbg."""
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", source)] + list(extra) + [
        "-L", LIB_DIR, "-lbbg", "-Wl,-rpath," + LIB_DIR, "-o", str(out)]
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + p.stdout)
    return out


def write_scene(path, scene, pos, kind=0, mode=0, count=1, dt=None):
    """The input file of facade_advance.cpp for a scene dict and positions."""
    cols = scene.get("colliders", [])
    with open(path, "wb") as f:
        f.write(struct.pack("<4i", len(pos), kind, mode, count))
        f.write(struct.pack("<3d", float(scene["mass"]), float(scene["spacing"]),
                            float(scene["dt"] if dt is None else dt)))
        f.write(struct.pack("<3d", *map(float, scene["domain_min"])))
        f.write(struct.pack("<3d", *map(float, scene["domain_max"])))
        f.write(struct.pack("<i", len(cols)))
        for c in cols:
            box = c["type"] == "box"
            size = c["size"] if box else (c["radius"], 0.0, 0.0)
            f.write(struct.pack("<2i", 1 if box else 2, 1 if c.get("reverse") else 0))
            f.write(struct.pack("<3d", *map(float, c.get("center", (0.0, 0.0, 0.0)))))
            f.write(struct.pack("<3d", *map(float, size)))
        f.write(np.ascontiguousarray(pos, np.float64).tobytes())


def read_result(path, n):
    raw = open(path, "rb").read()
    a = np.frombuffer(raw[: 48 * n], np.float64).reshape(2, n, 3)
    return a[0], a[1], struct.unpack("<i", raw[48 * n: 48 * n + 4])[0]
