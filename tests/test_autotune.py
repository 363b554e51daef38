"""Host logic of the batched-QR autotuner (no device): size classes, padded
flop counts, the per-matrix choice by predicted time and the CTAs-per-SM
setting, and the batched workload's shape distribution."""
import importlib.util
import os

import numpy as np
import pytest

from hybrid3_gb300 import autotune as AT

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_classes_cover_every_column_count():
    seen = set()
    for n in range(1, 4097):
        seen.add(AT.class_of(n))
    assert seen == set(range(len(AT.CLASSES)))
    los = [lo for lo, _ in AT.CLASSES]
    his = [hi for _, hi in AT.CLASSES]
    assert los[0] == 1 and all(h + 1 == l for h, l in zip(his, los[1:]))


def test_flop_counts():
    assert AT.qr_flops(100, 100) == pytest.approx(2 * 100 ** 3 - 2 * 100 ** 3 / 3)
    # Q^T C for n reflectors of an m-row Q: sum over reflectors of 4 (m - j) nrhs
    m, n, k = 300, 120, 4
    assert AT.ormqr_flops(m, n, k) == pytest.approx(sum(4 * (m - j) * k for j in range(n)), rel=1e-2)
    assert AT.padded(96, 64) == 128 and AT.padded(128, 64) == 128
    assert AT.padded_flops(96, 64, 64, 4) == pytest.approx(AT.qr_flops(128, 64) + AT.ormqr_flops(128, 64, 4))


def table(rates1, rates2=None, ctas=1):
    classes = {}
    for c, r in enumerate(AT.CLASSES):
        classes[c] = {"rates": {1: dict(rates1), 2: dict(rates2 or {})}, "n_range": list(r), "sample": 1}
    return {"ctas": ctas, "classes": classes}


def test_choice_trades_padding_against_rate():
    t = table({(96, 32): 0.5, (128, 32): 0.6})
    # 192 x 192: no padding at 96, 256 x 256 at 128 (2.4x the flops): 96 wins
    assert AT.choose(t, 192, 192, 4) == (96, 32)
    # 256 x 256: no padding at 128 (faster), 288 x 288 at 96: 128 wins
    assert AT.choose(t, 256, 256, 4) == (128, 32)
    assert AT.predicted_time(t, 256, 256, 4) == pytest.approx(AT.padded_flops(256, 256, 128, 4) / 0.6)


def test_choice_uses_the_tables_ctas_setting():
    t = table({(128, 32): 0.5}, {(128, 16): 0.9}, ctas=2)
    assert AT.choose(t, 256, 256, 4) == (128, 16)
    t["ctas"] = 1
    assert AT.choose(t, 256, 256, 4) == (128, 32)


def test_fixed_table_and_description():
    t = AT.fixed_table(64, 16, 2)
    assert t["ctas"] == 2
    for m, n in ((64, 32), (2048, 2048), (500, 300)):
        assert AT.choose(t, m, n, 4) == (64, 16)
    d = AT.describe(table({(64, 16): 0.25}, {(64, 16): 0.3}))
    assert d["ctas_per_sm"] == 1
    assert d["classes"]["0"]["padded_tflops"] == {"64/16/1": 0.25, "64/16/2": 0.3}


def test_batched_workload_shapes():
    spec = importlib.util.spec_from_file_location("bench", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    m, n = bench.batch_shapes(4096, 20151130)
    m, n = np.array(m), np.array(n)
    assert len(m) == 4096
    assert m.min() >= 64 and m.max() <= 2048 and np.all(m % 32 == 0)
    assert n.min() >= 32 and np.all(n <= m) and np.all(n % 32 == 0)
    # both ends of the ranges occur, and the draw is reproducible
    assert m.min() == 64 and m.max() == 2048 and n.min() == 32
    m2, n2 = bench.batch_shapes(4096, 20151130)
    assert np.array_equal(m, m2) and np.array_equal(n, n2)


def test_table_save_and_load_round_trip(tmp_path):
    t = table({(96, 16): 0.5, (128, 32): 0.6}, {(128, 16): 0.9}, ctas=2)
    path = tmp_path / "tune.json"
    AT.save(t, str(path))
    u = AT.load(str(path))
    assert u == t
    for m, n in ((192, 192), (2048, 1024), (64, 32)):
        assert AT.choose(u, m, n, 4) == AT.choose(t, m, n, 4)


def test_batch_layout():
    m, n, nb = [96, 64, 2048], [32, 64, 1000], [64, 32, 128]
    Mp, Np, a_off, t_off, c_off = AT.layout(m, n, nb, 4)
    assert Mp == [128, 64, 2048] and Np == [64, 64, 1024]
    assert list(a_off) == [0, 128 * 64, 128 * 64 + 64 * 64, 128 * 64 + 64 * 64 + 2048 * 1024]
    assert list(t_off) == [0, 2 * 1 * 64, 128 + 2 * 2 * 32, 128 + 128 + 16 * 8 * 128]
    # 4 right-hand sides take one tile column of NB
    assert list(c_off) == [0, 128 * 64, 128 * 64 + 64 * 32, 128 * 64 + 64 * 32 + 2048 * 128]
    # every offset is a whole number of 8-byte elements, tiles start on 16-byte boundaries
    assert all(int(x) % 2 == 0 for x in a_off)
