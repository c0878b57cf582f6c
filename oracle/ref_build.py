"""Build recipe for ``oracle/_ref/libref_kernels.so`` -- TEST INFRASTRUCTURE ONLY.

Compiles the reference's own per-thread device code for the host, unchanged, so the oracle can
be checked against the reference's arithmetic:

* ``K-SVD/K-SVD/OMP.cu`` from ``backsubst_Lt`` to the end of ``parOMP`` (lines 126-404: the
  Batch-OMP kernel and its helpers), and
* ``K-SVD/K-SVD/Multiplication.cu`` from ``device_A_times_x_modified`` to the end
  (lines 177-224: the per-atom ``a = Y_j - D v + d_j ||gamma_j||^2`` and coefficient kernels).

The two ranges are copied byte for byte from a reference checkout into the git-ignored folder
``oracle/_ref/`` and compiled with g++ against ``oracle/ref_shim.cpp`` (which defines the CUDA
qualifiers away and emulates the thread coordinates).  The reference checkout is read only here;
when it is absent (e.g. on a machine without it) ``build()`` returns None and the tests that
need the compiled reference skip.  The reference's build system (MSBuild, CUDA 8, MATLAB SDK) is
not used: these two ranges need none of it.

  python oracle/ref_build.py [REFERENCE_ROOT]      (default: $KSVD_REFERENCE or /root/reference)
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB_PATH = os.path.join(OUT_DIR, "libref_kernels.so")
SHIM = os.path.join(HERE, "ref_shim.cpp")
DEFAULT_ROOT = os.environ.get("KSVD_REFERENCE", "/root/reference")

# (source file, first line that starts the copied range, output name); ranges run to EOF
RANGES = [
    ("K-SVD/K-SVD/OMP.cu", "void backsubst_Lt(", "ref_omp_src.inc"),
    ("K-SVD/K-SVD/Multiplication.cu", "__global__ void device_A_times_x_modified(",
     "ref_mult_src.inc"),
]


def _extract(root: str):
    """Copies the ranges into OUT_DIR; returns a digest of what was copied."""
    h = hashlib.sha256()
    for rel, marker, out in RANGES:
        with open(os.path.join(root, rel), "r", encoding="utf-8", errors="replace") as f:
            lines = f.read().splitlines(keepends=True)
        start = next(i for i, l in enumerate(lines) if l.startswith(marker))
        # OMP.cu: the qualifier line just above the function belongs to it
        if start > 0 and lines[start - 1].strip() == "__inline__ __device__":
            start -= 1
        text = "".join(lines[start:])
        h.update(rel.encode() + b"\0" + text.encode())
        path = os.path.join(OUT_DIR, out)
        tmp = path + ".tmp%d" % os.getpid()
        with open(tmp, "w", encoding="utf-8") as f:
            f.write(text)
        os.replace(tmp, path)
    return h.hexdigest()


def available(root: str = DEFAULT_ROOT) -> bool:
    return all(os.path.exists(os.path.join(root, rel)) for rel, _, _ in RANGES)


def build(root: str = DEFAULT_ROOT, force: bool = False):
    """Compile the reference kernels for the host; None when no reference checkout is present
    (an already built library is still returned)."""
    if not available(root):
        return LIB_PATH if os.path.exists(LIB_PATH) else None
    os.makedirs(OUT_DIR, exist_ok=True)
    digest = _extract(root)
    with open(SHIM, "rb") as f:
        digest += hashlib.sha256(f.read()).hexdigest()
    stamp = os.path.join(OUT_DIR, "build.stamp")
    if not force and os.path.exists(LIB_PATH) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-fno-fast-math", "-ffp-contract=off",
           "-w", "-I", OUT_DIR, SHIM, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB_PATH


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_ROOT, force=True))
