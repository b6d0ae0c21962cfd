"""Recipe: build the reference's own SPH/PCISPH CPU path host-only, for pinning the oracle.

Test infrastructure only.  Compiles the hot-path sources where they lie under the
reference checkout (never copied into this repository) with g++, against the shim
headers in oracle/ref/shim/ (a host stand-in for the CUDA runtime, viewer stubs), plus
two headers generated into oracle/_ref/ from the reference's own:
  - cutil.h with its two `<<<grid, block>>>` launches rewritten as serial host loops;
  - geometry.h with `typedef float Float` (the FP32 variant; FP64 is as shipped).
Outputs only under oracle/_ref/ (git-ignored): libbbref_f64.so, libbbref_f32.so.  The
reference is x86-64 here; on a machine without the reference checkout nothing is built.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
SHIM = os.path.join(HERE, "shim")
REF = os.environ.get("BUBBLES_REFERENCE", "/root/reference")
SRC = os.path.join(REF, "src")

INC = ["core", "shapes", "third", "third/graphy", "cuda", "tests", "apps", "reconstruction",
       "boundaries"]
SOURCES = [
    "equations/sph_equations3.cpp", "equations/pcisph_equations3.cpp",
    "solvers/sph_solver3.cpp", "solvers/pcisph_solver3.cpp",
    "core/kernel.cpp", "core/particle.cpp", "core/collider.cpp", "core/shape.cpp",
    "core/point_generator.cpp", "core/statics.cpp", "core/util.cpp", "core/emitter.cpp",
    "core/transform.cpp", "core/quaternion.cpp", "cuda/cutil.cpp", "cuda/memory.cpp",
    "shapes/sphere.cpp", "shapes/box.cpp", "shapes/sphere2.cpp", "shapes/rectangle2.cpp",
    "shapes/bvh.cpp", "generator/bcclattice.cpp", "generator/triangle.cpp",
    "equations/sph_equations2.cpp", "third/serializer.cpp", "third/obj_loader.cpp",
    "reconstruction/marching_cubes.cpp", "apps/surface.cpp", "third/ply_loader.cpp",
]
LAUNCH = re.compile(r"(\w+)<<<\s*([^,>]+?)\s*,\s*([^>]+?)\s*>>>\s*\((.*)\);")


def available():
    return os.path.isdir(SRC)


def lib_path(variant):
    return os.path.join(OUT, "libbbref_%s.so" % variant)


def _host_loop(m):
    fn, grid, block, args = m.groups()
    return ("for(int bb_b = 0; bb_b < (int)(%s); bb_b++) for(int bb_t = 0; bb_t < (int)(%s); bb_t++)"
            "{ blockIdx.x = bb_b; threadIdx.x = bb_t; blockDim.x = (%s); gridDim.x = (%s); %s(%s); }"
            % (grid, block, block, grid, fn, args))


def generate(variant):
    gen = os.path.join(OUT, "gen_" + variant)
    os.makedirs(gen, exist_ok=True)
    text = open(os.path.join(SRC, "cuda", "cutil.h")).read()
    new, count = LAUNCH.subn(_host_loop, text)
    if count != 2:
        raise RuntimeError("expected two kernel launches in cutil.h, found %d" % count)
    open(os.path.join(gen, "cutil.h"), "w").write(new)
    if variant == "f32":
        geo = open(os.path.join(SRC, "core", "geometry.h")).read()
        flipped = geo.replace("//typedef float Float;\ntypedef double Float;", "typedef float Float;")
        if flipped == geo:
            raise RuntimeError("Float typedef not found in geometry.h")
        open(os.path.join(gen, "geometry.h"), "w").write(flipped)
    return gen


def build(force=False, verbose=False):
    if not available():
        return []
    os.makedirs(OUT, exist_ok=True)
    outs = []
    for variant in ("f64", "f32"):
        target = lib_path(variant)
        deps = [os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith((".cpp", ".py"))]
        deps += [os.path.join(SHIM, f) for f in os.listdir(SHIM)]
        if (not force and os.path.exists(target)
                and os.path.getmtime(target) >= max(os.path.getmtime(d) for d in deps)):
            outs.append(target)
            continue
        gen = generate(variant)
        objdir = os.path.join(OUT, "obj_" + variant)
        os.makedirs(objdir, exist_ok=True)
        flags = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-w",
                 "-pthread", "-I", gen, "-I", SHIM] + sum([["-I", os.path.join(SRC, d)] for d in INC], [])
        jobs = []
        for src in SOURCES + ["@ref_driver.cpp", "@shim_runtime.cpp"]:
            path = os.path.join(HERE, src[1:]) if src.startswith("@") else os.path.join(SRC, src)
            obj = os.path.join(objdir, os.path.basename(src).replace(".cpp", ".o").lstrip("@"))
            cmd = flags + ["-x", "c++", "-c", path, "-o", obj]
            jobs.append((obj, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        errors = []
        for obj, cmd, p in jobs:
            log = p.communicate()[0].decode()
            if p.returncode != 0:
                errors.append(" ".join(cmd[-4:]) + "\n" + log[-4000:])
        if errors:
            raise RuntimeError("reference host build failed:\n" + "\n".join(errors))
        link = ["g++", "-shared", "-pthread", "-o", target] + [o for o, _, _ in jobs]
        p = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if p.returncode != 0:
            raise RuntimeError("reference link failed:\n" + p.stdout.decode()[-4000:])
        outs.append(target)
    return outs


if __name__ == "__main__":
    print("\n".join(build(force="--force" in sys.argv, verbose=True)) or "reference not present")
