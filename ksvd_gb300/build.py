"""Build recipe for libksvd_gb300.so (sm_103a only, no CMake).

Every ``csrc/*.cu`` translation unit is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo`` and linked into
``ksvd_gb300/_build/libksvd_gb300.so`` (in-tree, git-ignored).  The library exports only the C ABI
declared in ``include/ksvd_gb300.h``.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libksvd_gb300.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)
CLI_SRC = os.path.join(HERE, "cli", "ksvd_cli.cpp")
CLI_PATH = os.path.join(OUT_DIR, "ksvd")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the K-SVD library needs the CUDA toolkit to build")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(ROOT, "include", "ksvd_gb300.h"))
    return sorted(hs)


def _fingerprint(flags):
    h = hashlib.sha256()
    for p in _sources() + _headers() + [CLI_SRC]:
        with open(p, "rb") as f:
            h.update(p.encode() + b"\0" + f.read())
    h.update(" ".join(flags).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    """Compile the library if its sources changed; returns the path of the shared object."""
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    cflags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-fvisibility=hidden", "--expt-relaxed-constexpr",
                     "-I", os.path.join(ROOT, "include")] + list(extra_flags)
    stamp = os.path.join(OUT_DIR, "build.stamp")
    fp = _fingerprint(cflags)
    if not force and os.path.exists(LIB_PATH) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == fp:
                return LIB_PATH
    objs = []

    def compile_one(src):
        obj = os.path.join(OUT_DIR, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc] + cflags + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = [nvcc] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs + [
        "-Xlinker", "-rpath=/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB_PATH)
    build_cli(nvcc)
    with open(stamp, "w") as f:
        f.write(fp)
    return LIB_PATH


def build_cli(nvcc=None) -> str:
    """The ``ksvd`` command-line program (host C++ over the library), next to the library."""
    nvcc = nvcc or _nvcc()
    tmp = CLI_PATH + ".tmp%d" % os.getpid()
    cmd = [nvcc, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), CLI_SRC, "-o", tmp,
           "-L", OUT_DIR, "-lksvd_gb300", "-cudart", "shared",
           "-Xlinker", "-rpath=$ORIGIN", "-Xlinker", "-rpath=/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("CLI build failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, CLI_PATH)
    return CLI_PATH


if __name__ == "__main__":
    import time

    t = time.time()
    print(build(force=True, verbose=True), "%.1fs" % (time.time() - t))
