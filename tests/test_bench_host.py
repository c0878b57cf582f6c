"""Host-side pieces of bench.py that need no GPU: the per-stage byte and flop counts, the rule
for the windowed list preparation (the library's rule restated), the affine CPU extrapolation,
and that the recorded ncu traffic constants belong to the Batch-OMP source as it is now (a
change to csrc/omp.cu needs a new counters capture, or the bench reports no traffic)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


class Shape:
    def __init__(self, n, K, T):
        self.n, self.K, self.T = n, K, T


def test_stage_counts_at_the_headline_shape():
    import bench

    c = Shape(256, 1024, 16)
    N = 1_000_000
    assert bench.stage_bytes(c, N, "omp") == N * (1024 * 4 + 16 * 8 + 4)
    assert bench.stage_bytes(c, N, "error") == N * 256 * 4 + N * 16 * 8 + N * 4
    # X is 1 GB: the preparation reads it once per window, not once per list entry
    assert bench.windowed_prep(256, 16, N)
    assert bench.stage_bytes(c, N, "lists") < N * 16 * 256 * 4 / 4
    assert bench.stage_flops(c, N, "omp") == float(N) * 1024 * 16 * 17
    assert bench.stage_flops(c, N, "dtx") == 2.0 * 256 * 1024 * N


@pytest.mark.parametrize("n,T,N,windowed", [
    (256, 16, 1_000_000, True),    # X = 1 GB
    (64, 4, 400_000, True),        # X = 102 MB, just above 96 MiB
    (64, 8, 10_000, False),        # X fits L2
    (256, 20, 1_000_000, False),   # T > 16: warp-per-entry preparation
    (250, 8, 1_000_000, False),    # n % 4 != 0
    (512, 8, 1_000_000, False),    # n > 256
])
def test_windowed_preparation_rule(n, T, N, windowed):
    import bench

    assert bench.windowed_prep(n, T, N) == windowed


def test_affine_cpu_extrapolation():
    import bench

    # t = 0.2 + 1e-5 N: two samples give the line back
    t = lambda n: 0.2 + 1e-5 * n
    assert bench.cpu_time_at(1_000_000, 50_000, t(50_000), 200_000, t(200_000)) == \
        pytest.approx(t(1_000_000))
    # one sample, or a fit that is not increasing: linear from the larger sample
    assert bench.cpu_time_at(1_000_000, 50_000, 1.0, None, None) == pytest.approx(20.0)
    assert bench.cpu_time_at(1_000_000, 50_000, 1.0, 200_000, 0.9) == pytest.approx(4.5)


def test_recorded_traffic_belongs_to_the_current_batch_omp_source():
    import bench

    fp = bench.source_fingerprint("omp")
    assert any(k[4] == fp for k in bench.MEASURED_OMP), (
        "csrc/omp.cu changed since the recorded ncu traffic: capture the counters again")
    assert fp in bench.MEASURED_BATCHED
