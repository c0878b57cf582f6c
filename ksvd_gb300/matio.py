"""Raw matrix files of the ``ksvd`` command-line program, and conversion to and from MATLAB
MAT-files (scipy.io, MAT v4/v5/v7 -- not the HDF5-based v7.3).

The reference reads ``input/X.mat`` (variable ``X``) and ``input/D.mat`` (variable ``D``) and
writes ``output/temp.mat`` (variable ``CUDA_Gamma``, K x N, double) through the MATLAB SDK
(K-SVD/K-SVD/FileManager.cu:98-160, main.cu:133-142).  The CLI reads and writes a plain format
instead:

    8 bytes  b"KSVDRAW1"
    uint32   dtype (0 float32, 1 float64)
    uint32   0
    uint64   rows
    uint64   cols
    rows x cols values, column-major, little-endian

Command line::

    python -m ksvd_gb300.matio mat2raw input/X.mat X X.raw
    python -m ksvd_gb300.matio raw2mat Gamma.raw output/temp.mat CUDA_Gamma
"""
from __future__ import annotations

import struct
import sys

import numpy as np

MAGIC = b"KSVDRAW1"
_DTYPES = {0: np.dtype("<f4"), 1: np.dtype("<f8")}

__all__ = ["write_raw", "read_raw", "mat_to_raw", "raw_to_mat"]


def write_raw(path, A, dtype=np.float32):
    """Write the 2-D array A (any layout) column-major as float32 or float64."""
    A = np.asarray(A)
    if A.ndim == 1:
        A = A[:, None]
    if A.ndim != 2:
        raise ValueError("raw files hold 2-D matrices")
    dt = np.dtype(dtype)
    code = {np.dtype(np.float32): 0, np.dtype(np.float64): 1}.get(dt)
    if code is None:
        raise ValueError("raw files hold float32 or float64")
    with open(path, "wb") as f:
        f.write(MAGIC + struct.pack("<IIQQ", code, 0, A.shape[0], A.shape[1]))
        f.write(np.asfortranarray(A, dtype=_DTYPES[code]).tobytes(order="F"))


def read_raw(path):
    """The matrix in a raw file (column-major numpy array of its stored type)."""
    with open(path, "rb") as f:
        head = f.read(32)
        if len(head) != 32 or head[:8] != MAGIC:
            raise ValueError("%s is not a KSVDRAW1 file" % path)
        code, _, rows, cols = struct.unpack("<IIQQ", head[8:])
        if code not in _DTYPES:
            raise ValueError("%s: unknown dtype code %d" % (path, code))
        data = np.frombuffer(f.read(), dtype=_DTYPES[code])
    if data.size != rows * cols:
        raise ValueError("%s: expected %d values, found %d" % (path, rows * cols, data.size))
    return data.reshape((rows, cols), order="F")


def mat_to_raw(mat_path, var, raw_path, dtype=np.float32):
    """Variable ``var`` of a MAT-file into a raw file."""
    from scipy.io import loadmat

    m = loadmat(mat_path)
    if var not in m:
        raise KeyError("%s has no variable %r (has %s)" % (mat_path, var,
                                                          sorted(k for k in m if k[0] != "_")))
    write_raw(raw_path, np.asarray(m[var], dtype=np.float64), dtype)


def raw_to_mat(raw_path, mat_path, var):
    """A raw file into a MAT-file as double variable ``var``."""
    from scipy.io import savemat

    savemat(mat_path, {var: np.asarray(read_raw(raw_path), dtype=np.float64)})


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) == 4 and argv[0] == "mat2raw":
        mat_to_raw(argv[1], argv[2], argv[3])
    elif len(argv) == 4 and argv[0] == "raw2mat":
        raw_to_mat(argv[1], argv[2], argv[3])
    else:
        print(__doc__.split("Command line::")[1].strip())
        return 2
    return 0


if __name__ == "__main__":
    sys.exit(main())
