"""Build libvkhel.so (sm_103a) and the CPU oracle library.

    python -m vkhel_gb300.build            # incremental
    python -m vkhel_gb300.build --force

Sources are compiled in parallel: CUDA translation units with nvcc for
``-gencode arch=compute_103a,code=sm_103a`` only, C files with the host C
compiler.  The link applies the vkhel version script (every ``vkhel_*``
symbol global, everything else local) and links the CUDA runtime statically,
so the library is self-contained.  Outputs go to ``vkhel_gb300/_build/``.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libvkhel.so")
ORACLE_LIB = os.path.join(ROOT, "oracle", "_build", "liboracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
                     "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]
CC_FLAGS = ["-O2", "-std=gnu11", "-fPIC", "-pthread", "-Wall", "-Wextra", "-Wno-unused-parameter",
            "-I" + os.path.join(ROOT, "include")]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    c = sorted(f for f in os.listdir(CSRC) if f.endswith(".c"))
    return cu, c


def _headers_mtime():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    inc = os.path.join(ROOT, "include", "vkhel")
    hs += [os.path.join(inc, f) for f in os.listdir(inc)]
    return max(os.path.getmtime(h) for h in hs)


def _stale(obj, src, hdr_mtime):
    return (not os.path.exists(obj) or os.path.getmtime(obj) < os.path.getmtime(src)
            or os.path.getmtime(obj) < hdr_mtime)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build_library(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    cu, c = _sources()
    hdr = _headers_mtime()
    jobs = []
    objs = []
    for f in cu:
        src, obj = os.path.join(CSRC, f), os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, src, hdr):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj])
    cc = os.environ.get("CC", "gcc")
    for f in c:
        src, obj = os.path.join(CSRC, f), os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, src, hdr):
            jobs.append([cc] + CC_FLAGS + ["-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    if force or jobs or not os.path.exists(LIB):
        syms = os.path.join(PKG, "vkhel.syms")
        _run([nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs +
             ["-Xlinker", "--version-script=" + syms, "-Xlinker", "--no-undefined", "-lpthread", "-ldl", "-lrt"])
    return LIB


def build_oracle():
    _run(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    return ORACLE_LIB


def main(argv):
    force = "--force" in argv
    print(build_library(force=force, verbose=True))
    print(build_oracle())


if __name__ == "__main__":
    main(sys.argv[1:])
