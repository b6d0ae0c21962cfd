"""In-tree build of libbbg.so (the CUDA kernels + C ABI) for sm_103a.

Each translation unit is compiled in parallel; the shared library lands in
``bubbles_gb300/_lib/libbbg.so``.  No cmake, one -gencode, no CPU fallback.
"""
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB_DIR = os.path.join(PKG, "_lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
INCLUDE = os.path.join(ROOT, "include")
LIB_NAME = "libbbg.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
              "-ffp-contract=off", "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-I", INCLUDE,
             "-I", CSRC]

CU_SOURCES = ["grid.cu", "sph.cu", "mlp.cu", "frame.cu", "emit.cu", "sdf.cu", "mesh.cu", "boundary.cu", "surface.cu", "mc.cu", "api.cu", "api_batch.cu", "api_io.cu", "api_emit.cu", "api_post.cu", "noalloc.cu"]
CXX_SOURCES = ["host_math.cpp"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; bubbles_gb300 needs the CUDA toolkit to build")


def lib_path():
    return os.path.join(LIB_DIR, LIB_NAME)


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    files.append(os.path.abspath(__file__))
    return files


def up_to_date():
    out = lib_path()
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose=False, extra_nvcc=()):
    if not force and up_to_date():
        return lib_path()
    os.makedirs(OBJ_DIR, exist_ok=True)
    nv = nvcc()
    jobs = []
    for src in CU_SOURCES:
        obj = os.path.join(OBJ_DIR, src + ".o")
        cmd = [nv] + ARCH + NVCC_FLAGS + list(extra_nvcc) + ["-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append((obj, cmd))
    for src in CXX_SOURCES:
        obj = os.path.join(OBJ_DIR, src + ".o")
        cmd = ["g++"] + CXX_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append((obj, cmd))
    procs = [(obj, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
             for obj, cmd in jobs]
    errors = []
    for obj, cmd, p in procs:
        log = p.communicate()[0].decode()
        if p.returncode != 0:
            errors.append(" ".join(cmd) + "\n" + log)
        elif verbose and log.strip():
            print(log)
    if errors:
        raise RuntimeError("libbbg build failed:\n" + "\n".join(errors))
    tmp = lib_path() + ".tmp"
    link = [nv] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in jobs] + ["-lcudart_static", "-lrt",
                                                                          "-lpthread", "-ldl"]
    p = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if p.returncode != 0:
        raise RuntimeError("libbbg link failed:\n" + " ".join(link) + "\n" + p.stdout.decode())
    os.replace(tmp, lib_path())
    return lib_path()


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
