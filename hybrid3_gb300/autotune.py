"""Per-shape choice of the tile order NB and inner block IB for batched FP64
QR (hqr_batch_*), measured on the device.

The reference fixes NB and IB per run (main.c takes them from the command
line).  A batch of uneven shapes has no single best pair: small matrices want
small tiles (more tasks per matrix, less zero padding), large ones large tiles
(fewer scheduling passes per flop, faster update kernels).  The tuner splits
the workload's shapes into size classes by their column count n, and for each
class times every candidate (NB, IB) on a sample of the workload's own shapes
in that class, zero-padded to NB multiples as the batch runs them: the rate of
a candidate is the padded flops it executes per second.  Each matrix then
takes the candidate with the least predicted time, its own padded flops at
NB divided by its class's rate for that candidate -- so a 96 x 96 matrix can
take NB 96 where the class's other shapes take 128.
"""
from __future__ import annotations

import time

import numpy as np

# column-count classes (inclusive bounds) and the candidates tried in each
CLASSES = ((1, 160), (161, 448), (449, 1024), (1025, 1 << 30))
CANDIDATES = ((64, 16), (96, 16), (96, 32), (128, 16), (128, 32), (192, 32), (256, 32))


def class_of(n: int) -> int:
    for c, (lo, hi) in enumerate(CLASSES):
        if lo <= n <= hi:
            return c
    raise ValueError(n)


def padded(x: int, nb: int) -> int:
    return -(-x // nb) * nb


def qr_flops(m: int, n: int) -> float:
    return 2.0 * m * n * n - 2.0 * n ** 3 / 3.0


def ormqr_flops(m: int, n: int, nrhs: int) -> float:
    """C <- Q^T C for n reflectors of an m-row Q on nrhs columns."""
    return 2.0 * nrhs * n * (2.0 * m - n)


def layout(m, n, nb, nrhs: int):
    """Padded shapes and element offsets of a batch stored contiguously:
    matrix b is Mp[b] x Np[b] (m, n rounded up to nb[b]) at a_off[b], its TAU
    (MT * NT * NB) at t_off[b] and its right-hand sides (Mp[b] x
    ceil(nrhs / NB) * NB) at c_off[b]; each offset array has one more entry,
    the total."""
    Mp = [padded(a, b) for a, b in zip(m, nb)]
    Np = [padded(a, b) for a, b in zip(n, nb)]
    a_len = [mp * np_ for mp, np_ in zip(Mp, Np)]
    t_len = [(mp // b) * (np_ // b) * b for mp, np_, b in zip(Mp, Np, nb)]
    c_len = [mp * padded(nrhs, b) for mp, b in zip(Mp, nb)]
    off = lambda L: np.concatenate([[0], np.cumsum(L)]).astype(np.int64)
    return Mp, Np, off(a_len), off(t_len), off(c_len)


class BatchData:
    """Device buffers of one batch: matrices (zero-padded tile layout, each
    ceil(m/NB) x ceil(n/NB) tiles of NB), TAU, right-hand sides (ceil(m/NB)
    x ceil(nrhs/NB) tiles), with pristine copies of A and C, contiguous."""

    def __init__(self, H, torch, m, n, nb, ib, nrhs: int, seed: int):
        f64 = torch.float64
        self.m, self.n, self.nb, self.ib, self.nrhs = list(m), list(n), list(nb), list(ib), nrhs
        cnt = len(self.m)
        self.Mp, self.Np, self.a_off, self.t_off, self.c_off = layout(self.m, self.n, self.nb, nrhs)
        self.A0 = torch.zeros(int(self.a_off[-1]), dtype=f64, device="cuda")
        self.A = torch.empty_like(self.A0)
        self.TAU = torch.zeros(int(self.t_off[-1]), dtype=f64, device="cuda")
        self.C0 = torch.zeros(int(self.c_off[-1]), dtype=f64, device="cuda")
        self.C = torch.empty_like(self.C0)
        L = H.lib()
        # the conversions run on torch's current stream: the generated
        # temporaries are freed to torch's allocator on that stream, so a
        # conversion on another stream could read reused memory
        s = torch.cuda.current_stream().cuda_stream
        g = torch.Generator(device="cuda")
        for b in range(cnt):
            # entries uniform[-1, 1), seeded per matrix; column-major m x n and m x nrhs
            g.manual_seed(seed + b)
            x = torch.rand(self.n[b], self.m[b], dtype=f64, device="cuda", generator=g) * 2.0 - 1.0
            H.check(L.hqr_colmajor_to_tiles_padded(self.m[b], self.n[b], self.m[b], self.nb[b], x.data_ptr(),
                                                   self.A0.data_ptr() + 8 * int(self.a_off[b]), s), "to tiles")
            y = torch.rand(nrhs, self.m[b], dtype=f64, device="cuda", generator=g) * 2.0 - 1.0
            H.check(L.hqr_colmajor_to_tiles_padded(self.m[b], nrhs, self.m[b], self.nb[b], y.data_ptr(),
                                                   self.C0.data_ptr() + 8 * int(self.c_off[b]), s), "to tiles")
        torch.cuda.synchronize()
        base = lambda t, o: [t.data_ptr() + 8 * int(x) for x in o[:-1]]
        self.pa, self.pt, self.pc = base(self.A, self.a_off), base(self.TAU, self.t_off), base(self.C, self.c_off)
        self.flops = sum(qr_flops(a, b) + ormqr_flops(a, b, nrhs) for a, b in zip(self.m, self.n))

    def restore(self):
        self.A.copy_(self.A0, non_blocking=True)
        self.C.copy_(self.C0, non_blocking=True)

    def batch(self, H, ctas_per_sm: int = 0):
        return H.Batch(self.Mp, self.Np, self.nb, self.ib, max_nrhs=self.nrhs, ctas_per_sm=ctas_per_sm)


def padded_flops(m: int, n: int, nb: int, nrhs: int) -> float:
    mp, np_ = padded(m, nb), padded(n, nb)
    return qr_flops(mp, np_) + ormqr_flops(mp, np_, nrhs)


def tune_batch(H, torch, m, n, nrhs: int, candidates=CANDIDATES, sample_flops: float = 1.5e11,
               max_sample: int = 600, seed: int = 7):
    """Measured rates (padded TFLOP/s) of every candidate (NB, IB) per size
    class, with one and, where the tiles fit, two executor CTAs per SM, for a
    workload of shapes (m[b], n[b]); then the CTAs-per-SM setting (the same
    for the whole batch) whose best per-matrix choices predict the least
    total time.  Returns {"ctas": k, "classes": {class: {"n_range", "sample",
    "rates": {k: {(NB, IB): rate}}}}}."""
    rng = np.random.default_rng(seed)
    m, n = np.asarray(m), np.asarray(n)
    classes = {}
    stream = torch.cuda.Stream()
    for c, (lo, hi) in enumerate(CLASSES):
        idx = np.nonzero((n >= lo) & (n <= hi))[0]
        if idx.size == 0:
            continue
        rng.shuffle(idx)
        take, acc = [], 0.0
        for b in idx:
            take.append(b)
            acc += qr_flops(int(m[b]), int(n[b]))
            if acc >= sample_flops or len(take) >= max_sample:
                break
        sm, sn = m[take].tolist(), n[take].tolist()
        rates = {1: {}, 2: {}}
        for nb, ib in candidates:
            d = BatchData(H, torch, sm, sn, [nb] * len(sm), [ib] * len(sm), nrhs, 1000 + c)
            pf = sum(padded_flops(a, b, nb, nrhs) for a, b in zip(sm, sn))
            for ctas in (1, 2):
                try:
                    bt = d.batch(H, ctas)
                except RuntimeError:   # the tiles do not fit two CTAs per SM
                    continue
                try:
                    times = []
                    for rep in range(2):   # the first run uploads the task tables
                        with torch.cuda.stream(stream):
                            d.restore()
                        torch.cuda.synchronize()
                        t0 = time.perf_counter()
                        bt.geqrf(d.pa, d.pt, stream=stream.cuda_stream)
                        bt.ormqr_t(d.pa, d.pt, d.pc, nrhs, stream=stream.cuda_stream)
                        times.append(time.perf_counter() - t0)
                    rates[ctas][(nb, ib)] = pf / times[-1] / 1e12
                finally:
                    bt.close()
            del d
            torch.cuda.empty_cache()
        classes[c] = {"rates": rates, "n_range": [lo, hi], "sample": len(sm)}
    table = {"ctas": 1, "classes": classes}
    best = None
    for ctas in (1, 2):
        if not all(e["rates"][ctas] for e in classes.values()):
            continue
        table["ctas"] = ctas
        t = sum(predicted_time(table, int(a), int(b), nrhs) for a, b in zip(m, n))
        if best is None or t < best[0]:
            best = (t, ctas)
    table["ctas"] = best[1]
    return table


def fixed_table(nb: int, ib: int, ctas: int = 1):
    """A table that picks (nb, ib) for every shape."""
    return {"ctas": ctas, "classes": {c: {"rates": {ctas: {(nb, ib): 1.0}}, "n_range": list(r), "sample": 0}
                                      for c, r in enumerate(CLASSES)}}


def _best(table, m: int, n: int, nrhs: int):
    rates = table["classes"][class_of(n)]["rates"][table["ctas"]]
    k = min(rates, key=lambda k: padded_flops(m, n, k[0], nrhs) / rates[k])
    return k, padded_flops(m, n, k[0], nrhs) / rates[k]


def predicted_time(table, m: int, n: int, nrhs: int) -> float:
    return _best(table, m, n, nrhs)[1]


def choose(table, m: int, n: int, nrhs: int):
    """(NB, IB) for an m x n matrix: the least predicted time over its class's
    measured candidates at the table's CTAs per SM."""
    return _best(table, m, n, nrhs)[0]


def save(table, path: str) -> None:
    """Write a tune_batch table as JSON (to reuse it for the same shapes and
    device without measuring again)."""
    import json
    enc = {"ctas": table["ctas"],
           "classes": {str(c): {"n_range": e["n_range"], "sample": e["sample"],
                                "rates": {str(k): [[nb, ib, r] for (nb, ib), r in rs.items()]
                                          for k, rs in e["rates"].items()}}
                       for c, e in table["classes"].items()}}
    with open(path, "w") as f:
        json.dump(enc, f, indent=1)


def load(path: str):
    """A table written by save()."""
    import json
    with open(path) as f:
        enc = json.load(f)
    return {"ctas": int(enc["ctas"]),
            "classes": {int(c): {"n_range": e["n_range"], "sample": e["sample"],
                                 "rates": {int(k): {(int(nb), int(ib)): float(r) for nb, ib, r in rs}
                                           for k, rs in e["rates"].items()}}
                        for c, e in enc["classes"].items()}}


def describe(table):
    """A JSON-able summary of a tune_batch table."""
    return {"ctas_per_sm": table["ctas"],
            "classes": {str(c): {"n_range": e["n_range"], "sample": e["sample"],
                                 "padded_tflops": {f"{k[0]}/{k[1]}/{ctas}": round(v, 4)
                                                   for ctas, r in e["rates"].items() for k, v in r.items()}}
                        for c, e in table["classes"].items()}}


# ---------------------------------------------------------------------------
# Single matrices (hqr_plan_*): precision, NB and IB per shape
# ---------------------------------------------------------------------------
# The split precisions run one tile order (128, the engine's K); their inner
# block is 16 whatever IB says (FP64 panels narrowed for the tensor-core
# updates), so IB only matters for plain FP64.
SINGLE_CANDIDATES = (
    ("split", 128, 32),
    ("fp64", 128, 32), ("fp64", 192, 32), ("fp64", 256, 32), ("fp64", 256, 64),
    ("fp64", 384, 32), ("fp64", 512, 64),
)
# Precisions that give an FP64-level backward error; "fast" (10 of the 36
# slice products) is considered only when the caller allows it (least squares
# refined on the augmented system).
FP64_LEVEL = ("split", "fp64")


def single_flops(m: int, n: int, want_q: bool) -> float:
    """Algorithmic flops of one factorization, plus Q generation (the same
    count again: 4/3 n^3 each for a square matrix) when want_q."""
    f = qr_flops(m, n)
    return f + (2.0 * m * n * n - 2.0 * n ** 3 / 3.0) if want_q else f


def sample_shape(m: int, n: int, budget: float, want_q: bool, quantum: int = 1536):
    """The shape the candidates are timed on: (m, n) itself when its flops fit
    the budget, else the same aspect ratio scaled down to fit, in multiples of
    `quantum` (a multiple of every candidate tile order)."""
    f = single_flops(m, n, want_q)
    if f <= budget:
        return m, n
    s = (budget / f) ** (1.0 / 3.0)
    ms = max(quantum, int(m * s) // quantum * quantum)
    ns = max(quantum, int(n * s) // quantum * quantum)
    return min(ms, padded(m, quantum)), min(ns, padded(n, quantum))


def predicted_single(rates, m: int, n: int, want_q: bool):
    """{candidate: predicted seconds} for an m x n matrix: its flops zero-padded
    to the candidate's tile order over the candidate's measured rate."""
    return {k: single_flops(padded(m, k[1]), padded(n, k[1]), want_q) / (r * 1e12)
            for k, r in rates.items() if r > 0}


def choose_single(table, m: int, n: int, want_q: bool = True, allow=FP64_LEVEL):
    """(precision, NB, IB) for an m x n matrix: the least predicted time over
    the allowed candidates, with the rates measured on the table's shape
    nearest to (m, n) (log distance) for the same want_q."""
    entries = [e for e in table["shapes"] if bool(e["want_q"]) == bool(want_q)]
    if not entries:
        raise KeyError("no measured shape with want_q=%s" % want_q)
    e = min(entries, key=lambda e: (np.log(e["m"] / m)) ** 2 + (np.log(e["n"] / n)) ** 2)
    rates = {k: r for k, r in e["rates"].items() if k[0] in allow}
    if not rates:
        raise KeyError("no allowed candidate measured")
    t = predicted_single(rates, m, n, want_q)
    return min(t, key=t.get)


def tune_single(H, torch, m: int, n: int, want_q: bool = True, candidates=SINGLE_CANDIDATES,
                budget: float = 3e12, reps: int = 2, seed: int = 11):
    """Measured rates (TFLOP/s of padded flops) of every candidate (precision,
    NB, IB) on an m x n matrix, or on a scaled sample of it (sample_shape):
    one warm-up and `reps` timed runs of hqr_geqrf (+ hqr_make_q) per
    candidate on a uniform[-1, 1) matrix, CUDA events on the current stream.
    Returns {"shapes": [{"m", "n", "sample", "want_q", "rates": {cand: rate}}]}."""
    L = H.lib()
    f64 = torch.float64
    sm, sn = sample_shape(m, n, budget, want_q)
    prec_code = {"fp64": H.HQR_PREC_FP64, "split": H.HQR_PREC_OZAKI, "fast": H.HQR_PREC_OZAKI_FAST,
                 "fp32": H.HQR_PREC_FP32}
    rates = {}
    for cand in candidates:
        prec, nb, ib = cand
        mp, np_ = padded(sm, nb), padded(sn, nb)
        try:
            plan = H.Plan(mp, np_, nb, ib, prec_code[prec])
        except RuntimeError:   # shape or tile order not supported by this precision
            continue
        try:
            A0 = torch.empty(mp * np_, dtype=f64, device="cuda")
            H.check(L.hqr_fill_uniform(mp, np_, nb, seed, A0.data_ptr(), None), "hqr_fill_uniform")
            A = torch.empty_like(A0)
            tau = torch.zeros((mp // nb) * (np_ // nb) * nb, dtype=f64, device="cuda")
            Q = torch.empty(mp * np_, dtype=f64, device="cuda") if want_q else None
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            times = []
            for rep in range(reps + 1):
                A.copy_(A0)
                ev[0].record()
                H.check(L.hqr_geqrf(plan.h, A.data_ptr(), tau.data_ptr(), None), "hqr_geqrf")
                if want_q:
                    H.check(L.hqr_make_q(plan.h, Q.data_ptr(), A.data_ptr(), tau.data_ptr(), 1, None),
                            "hqr_make_q")
                ev[1].record()
                torch.cuda.synchronize()
                if rep > 0:
                    times.append(ev[0].elapsed_time(ev[1]) / 1e3)
            rates[cand] = single_flops(mp, np_, want_q) / min(times) / 1e12
        finally:
            plan.close()
            del A0
            torch.cuda.empty_cache()
    return {"shapes": [{"m": int(m), "n": int(n), "sample": [int(sm), int(sn)], "want_q": bool(want_q),
                        "rates": rates}]}


def merge_single(*tables):
    """One table holding every measured shape of the given tables."""
    return {"shapes": [e for t in tables for e in t["shapes"]]}


def save_single(table, path: str) -> None:
    import json
    enc = {"shapes": [dict(e, rates=[[k[0], k[1], k[2], r] for k, r in e["rates"].items()])
                      for e in table["shapes"]]}
    with open(path, "w") as f:
        json.dump(enc, f, indent=1)


def load_single(path: str):
    import json
    with open(path) as f:
        enc = json.load(f)
    return {"shapes": [dict(e, rates={(p, int(nb), int(ib)): float(r) for p, nb, ib, r in e["rates"]})
                       for e in enc["shapes"]]}
