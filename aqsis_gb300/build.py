"""Build the hider's shared library in-tree with nvcc (sm_103a only).

Every translation unit is compiled in parallel to an object file under
aqsis_gb300/_build/, then linked into aqsis_gb300/_build/libaqh.so.
-fmad=false keeps multiply-adds unfused so the hit tests, inverse bilinear,
compositing and filter sums round exactly like the reference's scalar code.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libaqh.so")
SOURCES = ["api.cu", "bin.cu", "sample.cu", "sample_mb.cu", "filter.cu", "noalloc.cu", "server.cu", "mpdump.cpp",
           "dspy_host.cpp"]
# display drivers built as their own libraries
DRIVERS = {"dspy_capture.cpp": os.path.join(OUT, "libaqh_dspy_capture.so")}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
              "-Xptxas", "-v"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: str, verbose: bool) -> tuple:
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", os.path.join(SRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, obj, r.returncode, r.stdout + r.stderr


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)] + [os.path.join(HERE, "..", "include", "aqh.h")]
    if not force and os.path.exists(LIB) and all(os.path.exists(lib) for lib in DRIVERS.values()):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    logs = []
    for src, obj, rc, log in results:
        logs.append("== %s ==\n%s" % (src, log))
        if rc != 0:
            raise RuntimeError("nvcc failed on %s:\n%s" % (src, log))
    with open(os.path.join(OUT, "ptxas.log"), "w") as f:
        f.write("\n".join(logs))
    objs = [r[1] for r in results]
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    for src, lib in DRIVERS.items():
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fvisibility=hidden", os.path.join(SRC, src), "-o", lib]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("display driver build failed:\n" + r.stdout + r.stderr)
    if verbose:
        print("\n".join(logs))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force=True))
