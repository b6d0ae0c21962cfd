"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/sph_oracle.c twice with gcc -- FP32 (``typedef float Float``) and
FP64 (``typedef double Float``) -- into ``oracle/_lib/``.  ``-ffp-contract=off``
keeps x86-64 and aarch64 bit-identical; the reference itself is compiled without
floating-point contraction on x86-64.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "_lib")
SRC = os.path.join(HERE, "sph_oracle.c")

VARIANTS = {
    "f32": "float",
    "f64": "double",
}


def lib_path(variant):
    return os.path.join(LIB_DIR, "liborc_%s.so" % variant)


def build(force=False, quiet=True):
    os.makedirs(LIB_DIR, exist_ok=True)
    deps = [SRC, os.path.join(HERE, "sph_oracle.h"), os.path.abspath(__file__)]
    newest = max(os.path.getmtime(d) for d in deps)
    procs = []
    for variant, ctype in VARIANTS.items():
        out = lib_path(variant)
        if not force and os.path.exists(out) and os.path.getmtime(out) >= newest:
            continue
        cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-pthread",
               "-ffp-contract=off", "-fno-fast-math", "-fno-strict-aliasing",
               "-D_GNU_SOURCE", "-DORC_FLOAT=%s" % ctype, "-o", out + ".tmp", SRC, "-lm"]
        procs.append((out, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                            stderr=subprocess.STDOUT)))
    for out, p in procs:
        log = p.communicate()[0].decode()
        if p.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + log)
        if log.strip() and not quiet:
            print(log)
        os.replace(out + ".tmp", out)
    return [lib_path(v) for v in VARIANTS]


if __name__ == "__main__":
    print("\n".join(build(force=True, quiet=False)))
