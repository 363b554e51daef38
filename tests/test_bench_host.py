"""bench.py's host logic on the CPU (no device): the algorithmic flop counts
the reported TFLOP/s are computed from, the clock record's parsing (median
SM clock, throttle reasons), the scaling of the committed DRAM capture, the
batched workload's shape distribution and the replica timing without a
process group."""
import importlib.util
import json
import os
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_host", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_flop_counts(bench):
    n = 16384
    assert bench.qr_flops(n, n) == pytest.approx(4.0 / 3.0 * n ** 3)
    # dorgqr with k = n: 4/3 n^3 square, the factorization's count thin
    assert bench.orgqr_flops(n, n, n) == pytest.approx(4.0 / 3.0 * n ** 3)
    assert bench.orgqr_flops(4 * n, n, n) == pytest.approx(bench.qr_flops(4 * n, n))
    assert bench.step_flops(n, n) == pytest.approx(8.0 / 3.0 * n ** 3)
    # the n = 16384 factorization count the roofline uses
    assert bench.qr_flops(n, n) == pytest.approx(5.864062014805334e12)


def test_least_squares_flop_counts(bench):
    m, n, k = 32768, 8192, 16
    qr = bench.qr_flops(m, n)
    solve = (4.0 * m * n - 2.0 * n * n + n * n) * k
    assert bench.lstsq_flops(m, n, k, 0) == pytest.approx(qr + solve)
    assert bench.lstsq_flops(m, n, k, 2) == pytest.approx(qr + 3 * solve + 2 * 2.0 * m * n * k)
    # augmented: x0 and r0, then per step two products with A, two Q
    # applications and two triangular solves
    step = (4.0 * m * n + 2 * (4.0 * m * n - 2.0 * n * n) + 2.0 * n * n) * k
    assert bench.lstsq_flops(m, n, k, 3, augmented=True) == pytest.approx(qr + solve + 2.0 * m * n * k + 3 * step)


class _FakeProc:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def _clock_record(bench, lines):
    s = bench.ClockSampler(0)
    fd, s.path = tempfile.mkstemp(suffix=".csv")
    with os.fdopen(fd, "w") as f:
        f.write("\n".join(lines) + "\n")
    s.proc = _FakeProc()
    return s.stop()


def test_clock_record_median_and_reasons(bench):
    rows = [f"0, {mhz}, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, {cap}"
            for mhz, cap in ((2070, "Not Active"), (2055, "Active"), (2070, "Not Active"))]
    rec = _clock_record(bench, rows + ["garbage line"])
    assert rec["sm_mhz"] == 2070.0 and rec["sm_max_mhz"] == 2070.0
    assert rec["reasons"] == ["sw_power_cap"] and rec["samples"] == 3
    rec = _clock_record(bench, ["0, 1400, 2070, 1200, 0x8, Active, Active, Not Active, Not Active"])
    assert rec["reasons"] == ["hw_slowdown", "hw_thermal_slowdown"]
    assert _clock_record(bench, [])["reasons"] == ["no samples"]


def test_traffic_scales_the_committed_capture_by_flops(bench):
    d = json.load(open(os.path.join(ROOT, "profiles", "dag_exec_kernel_split_traffic.json")))
    base = bench.load_traffic(d["n"], d["NB"], "split")
    assert base == d["dram_bytes_per_factor_launch"]
    assert bench.load_traffic(2 * d["n"], d["NB"], "split") == pytest.approx(8 * base, rel=1e-9)
    assert bench.load_traffic(4096, 128, "no-such-precision") is None


def test_batched_shapes_follow_the_workload(bench):
    m, n = bench.batch_shapes(4096, 7)
    m, n = np.array(m), np.array(n)
    assert len(m) == 4096 and (m % 32 == 0).all() and (n % 32 == 0).all()
    assert m.min() >= 64 and m.max() <= 2048 and n.min() >= 32 and (n <= m).all()
    assert bench.batch_shapes(4096, 7) == bench.batch_shapes(4096, 7)


def test_replica_timing_without_a_process_group(bench):
    assert bench.max_over_ranks(1.5, None) == 1.5
    assert bench.job_rate(3e12, 1.5, None) == pytest.approx(2e12)
