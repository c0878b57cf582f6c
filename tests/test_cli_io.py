"""The ksvd CLI's file formats (raw matrices, MAT-file conversion) and its argument handling,
on the CPU; the GPU run of the CLI is in test_gpu_cli.py."""
import os
import subprocess

import numpy as np
import pytest


def test_raw_round_trip(tmp_path):
    from ksvd_gb300 import matio

    A = np.random.default_rng(0).standard_normal((7, 5))
    for dt in (np.float32, np.float64):
        p = tmp_path / ("a_%s.raw" % np.dtype(dt).name)
        matio.write_raw(p, A, dt)
        B = matio.read_raw(p)
        assert B.dtype == dt and B.shape == (7, 5) and B.flags.f_contiguous
        np.testing.assert_array_equal(B, A.astype(dt))
    with open(tmp_path / "bad.raw", "wb") as f:
        f.write(b"NOTRAW00" + bytes(24))
    with pytest.raises(ValueError):
        matio.read_raw(tmp_path / "bad.raw")


def test_mat_round_trip(tmp_path):
    pytest.importorskip("scipy")
    from scipy.io import loadmat, savemat

    from ksvd_gb300 import matio

    X = np.random.default_rng(1).standard_normal((12, 40))
    savemat(tmp_path / "X.mat", {"X": X})
    matio.mat_to_raw(tmp_path / "X.mat", "X", tmp_path / "X.raw", np.float64)
    np.testing.assert_array_equal(matio.read_raw(tmp_path / "X.raw"), X)
    matio.raw_to_mat(tmp_path / "X.raw", tmp_path / "G.mat", "CUDA_Gamma")
    np.testing.assert_array_equal(loadmat(tmp_path / "G.mat")["CUDA_Gamma"], X)
    with pytest.raises(KeyError):
        matio.mat_to_raw(tmp_path / "X.mat", "D", tmp_path / "D.raw")


def test_reference_dictionary_converts(tmp_path):
    """The reference's recorded initial dictionary (S/input/D.mat, frozen as a fixture) goes through
    the raw format unchanged."""
    from ksvd_gb300 import matio

    D = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_D_300x9.npy"))
    matio.write_raw(tmp_path / "D.raw", D, np.float64)
    np.testing.assert_array_equal(matio.read_raw(tmp_path / "D.raw"), D)


def test_cli_usage(native_lib):
    from ksvd_gb300 import build

    r = subprocess.run([build.CLI_PATH, "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "usage: ksvd" in r.stdout
    r = subprocess.run([build.CLI_PATH, "X.raw"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2
