"""The C-ABI library builds, loads and exports exactly what include/ksvd_gb300.h declares;
host-only entry points work without a GPU (no compute calls here)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ksvd_gb300.h")


def header_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"KSVD_API\s+[\w\s\*]+?\b(ksvd_\w+)\s*\(", src)))


def test_header_declares_the_reference_surface():
    fns = header_functions()
    for need in ("ksvd_create", "ksvd_destroy", "ksvd_omp", "ksvd_iterate", "ksvd_status_string",
                 "ksvd_update_dictionary", "ksvd_error", "ksvd_clear_dict", "ksvd_normcols"):
        assert need in fns


def test_library_exports_every_declared_symbol(native_lib):
    from ksvd_gb300 import _native

    for name in header_functions():
        assert hasattr(native_lib, name), name
    assert sorted(_native.EXPORTS) == header_functions()
    out = subprocess.run(["nm", "-D", "--defined-only", _native.library_path()],
                         capture_output=True, text=True, check=True).stdout
    exported = sorted(l.split()[-1] for l in out.splitlines() if " T " in l and
                      l.split()[-1].startswith("ksvd_"))
    assert exported == header_functions()           # nothing else leaks out


def test_header_compiles_as_c():
    src = '#include "ksvd_gb300.h"\nint main(void){ksvd_params p; ksvd_default_params(&p); return p.T;}\n'
    r = subprocess.run(["gcc", "-std=c99", "-fsyntax-only", "-I", os.path.dirname(HEADER), "-x", "c", "-"],
                       input=src, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_struct_layouts_match_bindings(tmp_path):
    """The ctypes structures of the Python binding have the C header's layout: every field at
    the same offset and the same total size, so a change to either side is caught here."""
    import ctypes as C

    from ksvd_gb300 import _native

    structs = {"ksvd_params": _native.Params, "ksvd_tuning": _native.Tuning,
               "ksvd_problem": _native.Problem, "ksvd_stage_times": _native.StageTimes}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "ksvd_gb300.h"',
             'int main(void) {']
    for cname, py in structs.items():
        lines.append('printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines += ['return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c99", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in structs.items():
        assert got[(cname, "sizeof")] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_status_strings_and_defaults(native_lib):
    from ksvd_gb300._native import Params

    assert native_lib.ksvd_abi_version() == 1
    for s in range(8):
        assert native_lib.ksvd_status_string(s).decode()
    p = Params()
    native_lib.ksvd_default_params(C.byref(p))
    assert (p.T, p.use_thresh, p.max_replace_signals) == (6, 4, 5000)
    assert abs(p.mu_thresh - 0.8) < 1e-7


def test_random_permutation_host_only(native_lib):
    from ksvd_gb300 import random_permutation

    a = random_permutation(123, 0, 1024)
    b = random_permutation(123, 0, 1024)
    c = random_permutation(123, 1, 1024)
    assert np.array_equal(np.sort(a), np.arange(1024))
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert native_lib.ksvd_random_permutation(1, 0, 0, None) == 1


def test_create_rejects_bad_params(native_lib):
    from ksvd_gb300._native import Params

    p = Params()
    native_lib.ksvd_default_params(C.byref(p))
    h = C.c_void_p()
    p.n, p.K, p.T = 64, 2048, 8
    assert native_lib.ksvd_create(C.byref(h), C.byref(p), None) == 2   # K > 1024 unsupported
    p.K, p.T = 256, 100
    assert native_lib.ksvd_create(C.byref(h), C.byref(p), None) == 2   # T > 64
    p.T = 0
    assert native_lib.ksvd_create(C.byref(h), C.byref(p), None) == 1
    assert native_lib.ksvd_create(None, C.byref(p), None) == 1
    assert native_lib.ksvd_create(C.byref(h), None, None) == 1


def test_null_handle_calls_fail_cleanly(native_lib):
    assert native_lib.ksvd_omp(None, None, None, 0, None, None, None, None) == 1
    assert native_lib.ksvd_iterate(None, None, None, 1, 1, None, None, None, None, None) == 1
    assert native_lib.ksvd_synchronize(None) == 1
    native_lib.ksvd_destroy(None)
    assert native_lib.ksvd_workspace_bytes(None) == 0


def test_datagen_shapes():
    from ksvd_gb300 import datagen

    p = datagen.make_problem("cfg0", N=500)
    X, D = p["X"], p["D"]
    assert X.shape == (64, 500) and D.shape == (64, 256)
    assert X.flags.f_contiguous and X.dtype == np.float32
    np.testing.assert_allclose(np.linalg.norm(D, axis=0), 1.0, atol=1e-5)
    p1 = datagen.make_problem("cfg1", N=1000)
    np.testing.assert_allclose(p1["X"].mean(1), 0.0, atol=1e-5)      # row means removed
    q = datagen.make_problem("cfg0", N=500)
    assert np.array_equal(q["X"], X)                                  # seeded
