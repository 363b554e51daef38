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


# --- single matrices --------------------------------------------------------
def test_single_flops_match_the_bench_definition():
    # factorization + Q generation: 8/3 n^3 square; tall: twice 2 m n^2 - 2/3 n^3
    assert AT.single_flops(300, 300, True) == pytest.approx(8.0 / 3.0 * 300 ** 3)
    assert AT.single_flops(600, 200, True) == pytest.approx(2 * AT.qr_flops(600, 200))
    assert AT.single_flops(600, 200, False) == pytest.approx(AT.qr_flops(600, 200))


def test_sample_shape_keeps_the_aspect_and_the_budget():
    assert AT.sample_shape(2048, 2048, 1e12, True) == (2048, 2048)
    ms, ns = AT.sample_shape(16384, 16384, 3e12, True)
    assert ms == ns and ms % 1536 == 0
    assert AT.single_flops(ms, ns, True) <= 3e12
    ms, ns = AT.sample_shape(65536, 16384, 3e12, True)
    assert ms % 1536 == 0 and ns % 1536 == 0 and 3.0 <= ms / ns <= 5.0


def single_table(shapes):
    return {"shapes": [{"m": m, "n": n, "sample": [m, n], "want_q": q, "rates": r} for m, n, q, r in shapes]}


def test_single_choice_trades_padding_against_rate_and_respects_precision():
    rates = {("split", 128, 32): 10.0, ("fp64", 256, 32): 1.0, ("fp64", 192, 32): 0.9,
             ("fast", 128, 32): 13.0}
    t = single_table([(8192, 8192, True, rates)])
    # the fastest FP64-level candidate; "fast" only when allowed
    assert AT.choose_single(t, 8192, 8192) == ("split", 128, 32)
    assert AT.choose_single(t, 8192, 8192, allow=("split", "fp64", "fast")) == ("fast", 128, 32)
    # FP64 only: 192 x 192 padding to 256 costs 2.4x the flops, 192 wins at 0.9 vs 1.0
    assert AT.choose_single(t, 192, 192, allow=("fp64",)) == ("fp64", 192, 32)
    assert AT.choose_single(t, 256, 256, allow=("fp64",)) == ("fp64", 256, 32)
    with pytest.raises(KeyError):
        AT.choose_single(t, 8192, 8192, want_q=False)


def test_single_choice_takes_the_nearest_measured_shape():
    near = {("split", 128, 32): 2.0, ("fp64", 256, 32): 1.0}
    far = {("split", 128, 32): 0.1, ("fp64", 256, 32): 1.0}
    t = single_table([(2048, 2048, True, near), (32768, 32768, True, far)])
    assert AT.choose_single(t, 3072, 3072) == ("split", 128, 32)
    assert AT.choose_single(t, 24576, 24576) == ("fp64", 256, 32)


def test_single_table_round_trip(tmp_path):
    t = single_table([(4096, 1024, False, {("split", 128, 32): 3.5, ("fp64", 256, 64): 0.8})])
    p = str(tmp_path / "single.json")
    AT.save_single(t, p)
    u = AT.load_single(p)
    assert u["shapes"][0]["rates"] == t["shapes"][0]["rates"]
    assert AT.merge_single(t, u)["shapes"][1]["m"] == 4096
