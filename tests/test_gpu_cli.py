"""The ksvd CLI on the GPU: the reference executable's stdout contract, the same numbers as the
library call, checkpoint/resume continuing a run exactly, and row-mean removal."""
import re
import subprocess

import numpy as np
import pytest

from conftest import rel_rmse

pytestmark = pytest.mark.gpu

RMSE_LINE = re.compile(r"^Iteration (\d\d) / (\d+) complete, RMSE = ([0-9.]+)$", re.M)


def _files(tmp_path):
    from ksvd_gb300 import datagen, matio

    p = datagen.make_problem("cfg0", N=3000, dict_from="extra")
    matio.write_raw(tmp_path / "X.raw", p["X"], np.float32)
    matio.write_raw(tmp_path / "D.raw", p["D"], np.float32)
    return p


def _run(args):
    from ksvd_gb300 import build

    r = subprocess.run([build.CLI_PATH] + [str(a) for a in args], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_cli_matches_library_and_stdout_contract(cuda, tmp_path):
    import torch

    from ksvd_gb300 import Handle, matio

    p = _files(tmp_path)
    c = p["cfg"]
    out = _run(["-T", c.T, "--iters", 3, tmp_path / "X.raw", tmp_path / "D.raw",
                tmp_path / "G.raw", tmp_path / "Dout.raw"])
    lines = RMSE_LINE.findall(out)
    assert [(int(a), int(b)) for a, b, _ in lines] == [(1, 3), (2, 3), (3, 3)]
    assert "Final Execution Time =>\t\t" in out and out.rstrip().endswith("# Exiting!")
    assert "Dictionary size: 64 x 256" in out and "Input data size: 64 x 3000" in out
    h = Handle(c.n, c.K, c.T)
    X = torch.from_numpy(np.ascontiguousarray(np.asarray(p["X"], np.float32).T)).to(cuda)
    D = torch.from_numpy(np.ascontiguousarray(np.asarray(p["D"], np.float32).T)).to(cuda)
    idx, coef, nnz, rmse = h.iterate(D, X, 3)
    np.testing.assert_allclose([float(v) for _, _, v in lines], rmse, rtol=2e-4, atol=1e-5)
    G = matio.read_raw(tmp_path / "G.raw")
    assert G.shape == (c.K, 3000) and G.dtype == np.float64
    assert np.all((G != 0).sum(axis=0) <= c.T)
    assert rel_rmse(matio.read_raw(tmp_path / "Dout.raw"), D.double().cpu().numpy().T) <= 1e-3
    h.close()


def test_cli_checkpoint_resume_continues_the_run(cuda, tmp_path):
    from ksvd_gb300 import matio

    p = _files(tmp_path)
    T = p["cfg"].T
    full = _run(["-T", T, "--iters", 4, tmp_path / "X.raw", tmp_path / "D.raw",
                 tmp_path / "G1.raw", tmp_path / "D1.raw"])
    _run(["-T", T, "--iters", 2, "--checkpoint", tmp_path / "ck.bin", tmp_path / "X.raw",
          tmp_path / "D.raw", tmp_path / "G2.raw"])
    resumed = _run(["-T", T, "--iters", 4, "--resume", tmp_path / "ck.bin", tmp_path / "X.raw",
                    tmp_path / "D.raw", tmp_path / "G3.raw", tmp_path / "D3.raw"])
    a = {int(i): float(v) for i, _, v in RMSE_LINE.findall(full)}
    b = {int(i): float(v) for i, _, v in RMSE_LINE.findall(resumed)}
    assert sorted(b) == [3, 4]
    for k in (3, 4):
        assert abs(a[k] - b[k]) <= 2e-4 * a[k] + 1e-5
    assert rel_rmse(matio.read_raw(tmp_path / "D3.raw"), matio.read_raw(tmp_path / "D1.raw")) <= 1e-3


def test_remove_row_mean(cuda):
    import torch

    from ksvd_gb300 import Handle, datagen

    p = datagen.make_problem("cfg1", N=20000)
    X = np.asarray(p["X"], np.float64) + 3.0          # rows with clearly non-zero means
    Xd = torch.from_numpy(np.ascontiguousarray(X.T.astype(np.float32))).to(cuda)
    h = Handle(X.shape[0], 16, 4)
    mean = h.remove_row_mean(Xd)
    want = Xd.double().cpu().numpy()                   # (already centred on the device)
    np.testing.assert_allclose(mean.double().cpu().numpy(),
                               X.astype(np.float32).astype(np.float64).mean(axis=1), rtol=1e-6)
    assert np.abs(want.mean(axis=0)).max() <= 1e-5
    h.close()


def test_cli_error_target(cuda, tmp_path):
    """--eps: error-constrained coding through the CLI; every signal's code meets the target or
    uses T atoms."""
    from ksvd_gb300 import matio

    p = _files(tmp_path)
    X = np.asarray(p["X"], np.float64)
    eps = float(0.3 * np.median(np.linalg.norm(X, axis=0)))
    out = _run(["-T", 20, "--eps", eps, "--iters", 2, tmp_path / "X.raw", tmp_path / "D.raw",
                tmp_path / "G.raw", tmp_path / "Dout.raw"])
    assert len(RMSE_LINE.findall(out)) == 2
    G = matio.read_raw(tmp_path / "G.raw")
    D = matio.read_raw(tmp_path / "Dout.raw")
    counts = (G != 0).sum(axis=0)
    assert counts.max() <= 20 and counts.mean() < 20
