#!/usr/bin/env python3
"""Tiled Householder QR benchmark: factorization + explicit Q generation.

Workload (one step): A (n x n, i.i.d. uniform[-1,1) from a fixed seed, tile
layout, NB x NB tiles) is factored in place (Hybrid_tile_QR semantics) and the
explicit Q is generated (Hybrid_make_Q semantics: Q^T into a zeroed array, the
reflectors removed from A).  Throughput counts algorithmic flops only:
factorization 2mn^2 - 2n^3/3 plus Q generation (LAPACK dorgqr count with
k = n) 4mnk - 2(m+n)k^2 + 4k^3/3 -- 8/3 n^3 for a square matrix.

Arms:
  default            the GB300 library, inputs resident in HBM (`value`), and
                     the same workload end to end through the drop-in C entry
                     points with pinned host buffers (`e2e`)
  --impl reference   the reference's CPU implementation of the path on this
                     host's cores, on a bounded sample of the same workload

Multi-GPU (torchrun): one independent replica per GPU ("replicas only": the
path has no exchange step); value = all ranks' flops / max over ranks of time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "tile-QR TFLOP/s at FP64-level backward error: split-precision vs plain FP64"
DP = ctypes.POINTER(ctypes.c_double)


PRECISION_TEXT = {"split": "split (Ozaki BF16 slices on tcgen05, FP64 panels)",
                  "fast": "reduced split (the 10 slice products of weight <= 3 on tcgen05, FP64 panels)",
                  "fp32": "FP32-class (FP32 panel arithmetic, the reduced split updates)",
                  "fp64": "fp64 (plain)"}


def prec_code(H, precision: str) -> int:
    return {"split": H.HQR_PREC_OZAKI, "fast": H.HQR_PREC_OZAKI_FAST,
            "fp32": H.HQR_PREC_FP32}.get(precision, H.HQR_PREC_FP64)


def max_over_ranks(x: float, dist, device: str = "cuda") -> float:
    """The largest x over the ranks (x itself without a process group): the
    job's time is that of its slowest replica."""
    if not dist:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, seconds: float, dist, device: str = "cuda") -> float:
    """Whole-job throughput of independent replicas: every rank's units over
    the slowest rank's time."""
    world = dist.get_world_size() if dist else 1
    return world * units_per_rank / max_over_ranks(seconds, dist, device)


def qr_flops(m: int, n: int) -> float:
    return 2.0 * m * n * n - 2.0 * n ** 3 / 3.0


def orgqr_flops(m: int, n: int, k: int) -> float:
    return 4.0 * m * n * k - 2.0 * (m + n) * k * k + 4.0 * k ** 3 / 3.0


def step_flops(m: int, n: int) -> float:
    return qr_flops(m, n) + orgqr_flops(m, n, n)


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
# CPU baseline (the reference's algorithm on the host cores)
# ---------------------------------------------------------------------------
def cpu_sample(n: int, NB: int, IB: int, threads: int):
    """One factorization + Q generation of an n x n sample on the host.
    Uses the reference's own build when it can be loaded here, else the
    oracle's task-DAG restatement.  Returns (seconds, kind)."""
    import oracle as O
    A = O.to_tiles(O.uniform_matrix(n, n, 20151130), NB)
    kind = "port"
    if O.ref_available() and os.environ.get("OMP_NUM_THREADS", "").startswith("1,"):
        try:
            O.ref_lib()
            kind = "reference"
        except OSError:
            kind = "port"
    if kind == "reference":
        t0 = time.perf_counter()
        a, tau = O.ref_tile_qr(A, n, n, NB, IB)
        O.ref_make_Q(a, tau, n, n, NB, IB)
        return time.perf_counter() - t0, kind
    L = O.lib()
    L.orc_tile_qr_dag.restype = ctypes.c_int
    L.orc_tile_qr_dag.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_int, ctypes.c_int, DP, DP]
    L.orc_make_Q_dag.restype = None
    L.orc_make_Q_dag.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_int, DP, DP, DP]
    O.set_threads(threads)
    a = A.copy()
    tau = np.zeros((n // NB) ** 2 * NB)
    q = np.zeros(n * n)
    t0 = time.perf_counter()
    L.orc_tile_qr_dag(n, n, NB, IB, O.ptr(a), O.ptr(tau))
    L.orc_make_Q_dag(n, n, NB, O.ptr(q), O.ptr(a), O.ptr(tau))
    return time.perf_counter() - t0, kind


def run_reference(args, rank: int):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n = args.cpu_n
    nb = 256   # the reference's CPU configuration (NB = 256, IB = 32)
    for _ in range(args.warmup):
        cpu_sample(n, nb, args.ib, threads)
    times = []
    kind = "port"
    for _ in range(args.steps):
        t, kind = cpu_sample(n, nb, args.ib, threads)
        times.append(t)
    total = sum(times)
    value = args.steps * step_flops(n, n) / total / 1e12
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 6), "unit": "TFLOP/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * total / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"tiled QR + Q generation, sample n={n} of the n={args.n} "
                               f"workload, NB={nb}, IB={args.ib}, uniform[-1,1) seed 20151130",
                   "n": args.n, "sample_n": n, "NB": nb, "IB": args.ib},
        "cpu_baseline": {"value": round(value, 6), "unit": "TFLOP/s", "cores": threads,
                         "kind": kind, "sample": f"{n}x{n} factorization + make_Q per step"},
        "e2e": {"value": round(value, 6), "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# the GB300 arm
# ---------------------------------------------------------------------------
def load_traffic(n: int, NB: int, precision: str):
    """DRAM bytes per factorization launch from the committed ncu summary of
    that kernel (captured on a smaller case and scaled by the flop ratio)."""
    p = os.path.join(ROOT, "profiles", f"dag_exec_kernel_{precision}_traffic.json")
    if not os.path.exists(p):
        return None
    try:
        d = json.load(open(p))
        scale = qr_flops(n, n) / qr_flops(d["n"], d["n"])
        return int(d["dram_bytes_per_factor_launch"] * scale)
    except Exception:
        return None


def load_batch_traffic(qr_total: float):
    """DRAM bytes of a batched factorization launch, from the committed ncu
    summary of a 128-matrix case scaled by the algorithmic flop ratio."""
    p = os.path.join(ROOT, "profiles", "dag_exec_kernel_batch_traffic.json")
    try:
        d = json.load(open(p))
        return int(d["dram_bytes_per_factor_launch"] * qr_total / d["qr_flops"])
    except Exception:
        return None


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return json.load(open(p))
    except Exception:
        return {}


# slice products per emulated product: 8 digits per element, the 36 digit
# pairs with p + q <= 7 (NB = 128, the only tile order of the split path)
def split_products(NB: int) -> int:
    return 36


def graded_tiles(H, torch, L, n: int, NBs, kappa: float, seed: int):
    """A = U diag(sigma) V^T in the tile layouts of each NB in NBs, on the
    device: U, V Haar (QR of Gaussians with columns signed by diag(R),
    Mezzadri 2007), sigma_i = kappa^(-i/(n-1)).  Input generation only
    (torch, outside the timed path)."""
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)

    def haar():
        Z = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=gen)
        Q, R = torch.linalg.qr(Z)
        Q *= torch.sign(torch.diagonal(R))
        del Z, R
        return Q

    U = haar()
    U *= kappa ** (-torch.arange(n, dtype=torch.float64, device="cuda") / (n - 1))
    V = haar()
    A = U @ V.T
    del U, V
    cm = A.T.contiguous()          # column-major storage of A
    del A
    out = {}
    for NB in NBs:
        tiles = torch.empty(n * n, dtype=torch.float64, device="cuda")
        H.check(L.hqr_colmajor_to_tiles(n, n, NB, cm.data_ptr(), tiles.data_ptr(), None), "to tiles")
        out[NB] = tiles
    torch.cuda.synchronize()
    del cm
    torch.cuda.empty_cache()
    return out


def measure(H, torch, L, args, precision: str, n: int, NB: int, IB: int, steps: int, warmup: int,
            dist, world: int, clocks_too: bool, check: bool, init=None, rows=None):
    """Time `steps` device-resident steps (factorization + make_Q) of an
    rows x n matrix (square when rows is None).  init: the input in tile
    layout (device), else the seeded uniform matrix."""
    N = n
    M = rows or n
    ntau = (M // NB) * (N // NB) * NB
    prec = prec_code(H, precision)
    stream = torch.cuda.Stream()
    s = stream.cuda_stream
    f64 = torch.float64
    dA0 = torch.empty(M * N, dtype=f64, device="cuda")
    dA = torch.empty_like(dA0)
    dQ = torch.empty_like(dA0)
    dTAU = torch.zeros(ntau, dtype=f64, device="cuda")
    if init is None:
        H.check(L.hqr_fill_uniform(M, N, NB, 20151130, dA0.data_ptr(), s), "fill")
    else:
        dA0.copy_(init)
    plan = H.Plan(M, N, NB, IB, prec)
    if args.tree:
        plan.set_tree(args.tree)
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def step(rec=None):
        with torch.cuda.stream(stream):
            dA.copy_(dA0, non_blocking=True)
            if rec:
                rec[0].record(stream)
            H.check(L.hqr_geqrf_async(plan.h, dA.data_ptr(), dTAU.data_ptr(), s), "geqrf")
            if rec:
                rec[1].record(stream)
            dQ.zero_()
            if rec:
                rec[2].record(stream)
            H.check(L.hqr_make_q_async(plan.h, dQ.data_ptr(), dA.data_ptr(), dTAU.data_ptr(), 1, s),
                    "make_q")
            if rec:
                rec[3].record(stream)

    for _ in range(warmup):
        step()
    H.check(L.hqr_plan_status(plan.h, s), "warm-up run")
    clocks = ClockSampler(torch.cuda.current_device()) if clocks_too else None
    if clocks:
        clocks.start()
    recs = [[ev(), ev(), ev(), ev()] for _ in range(steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t_start, t_end = ev(), ev()
    with torch.cuda.stream(stream):
        t_start.record(stream)
    for r in recs:
        step(r)
    with torch.cuda.stream(stream):
        t_end.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop() if clocks else None
    H.check(L.hqr_plan_status(plan.h, s), "timed run")
    elapsed = max_over_ranks(t_start.elapsed_time(t_end) / 1e3, dist)
    fact_s = [r[0].elapsed_time(r[1]) / 1e3 for r in recs]
    mq_s = [r[2].elapsed_time(r[3]) / 1e3 for r in recs]
    stats_mq = plan.stats(s)
    acc = {}
    if check and M != N:
        # tall: Q^T I_{M x N} has orthonormal columns, and R^T R = A^T A
        f64 = torch.float64
        cm = torch.empty(M * N, dtype=f64, device="cuda")
        H.check(L.hqr_tiles_to_colmajor(M, N, NB, dQ.data_ptr(), cm.data_ptr(), s), "from tiles")
        torch.cuda.synchronize()
        X = cm.view(N, M).T
        acc["orth_fro"] = float(torch.linalg.norm(X.T @ X - torch.eye(N, dtype=f64, device="cuda")))
        torch.cuda.synchronize()
        H.check(L.hqr_tiles_to_colmajor(M, N, NB, dA0.data_ptr(), cm.data_ptr(), s), "from tiles")
        torch.cuda.synchronize()
        G = X.T @ X   # X now views A0
        Rt = torch.empty(M * N, dtype=f64, device="cuda")
        H.check(L.hqr_tiles_to_colmajor(M, N, NB, dA.data_ptr(), Rt.data_ptr(), s), "from tiles")
        torch.cuda.synchronize()
        R = torch.triu(Rt.view(N, M).T[:N])
        acc["gram_rel"] = float(torch.linalg.norm(R.T @ R - G) / torch.linalg.norm(G))
        del cm, X, G, Rt, R
    elif check:
        # ||A - Q R||_F / ||A||_F and ||I - Q Q^T||_F from the Q^T array of the last
        # step, on the device in FP64 (the checks of main.c:201-258)
        dW = torch.empty_like(dA0)
        r2 = ctypes.c_double()
        a2 = ctypes.c_double()
        H.check(L.hqr_dgemm_tn(N, NB, dQ.data_ptr(), dA.data_ptr(), dW.data_ptr(), s), "QR")
        H.check(L.hqr_frob2(M, N, NB, dW.data_ptr(), dA0.data_ptr(), 0.0, ctypes.byref(r2), s), "frob")
        H.check(L.hqr_frob2(M, N, NB, dA0.data_ptr(), None, 0.0, ctypes.byref(a2), s), "frob")
        acc["resid_fro_rel"] = float(np.sqrt(r2.value / a2.value))
        H.check(L.hqr_dgemm_tn(N, NB, dQ.data_ptr(), dQ.data_ptr(), dW.data_ptr(), s), "QQt")
        H.check(L.hqr_frob2(M, N, NB, dW.data_ptr(), None, 1.0, ctypes.byref(r2), s), "frob")
        acc["orth_fro"] = float(np.sqrt(r2.value))
        del dW
    # task counts of the factorization (run one more, untimed, for its stats)
    step()
    torch.cuda.synchronize()
    plan.close()
    del dA0, dA, dQ, dTAU
    torch.cuda.empty_cache()
    return {"elapsed": elapsed, "fact_s": fact_s, "mq_s": mq_s, "acc": acc, "clocks": clk,
            "stats_mq": stats_mq, "flops": step_flops(M, N) * steps * world}


class HostArrays:
    """Page-locked host arrays from the library's allocator (hqr_host_alloc,
    cudaHostAlloc): the arrays a caller of the drop-in entry points hands over."""

    def __init__(self, L, torch):
        self.L, self.torch, self.ptrs = L, torch, []

    def empty(self, count: int):
        p = ctypes.c_void_p()
        rc = self.L.hqr_host_alloc(ctypes.byref(p), ctypes.c_size_t(count * 8))
        if rc != 0:
            raise MemoryError(f"hqr_host_alloc of {count * 8} bytes failed ({rc})")
        self.ptrs.append(p.value)
        return self.torch.from_numpy(np.ctypeslib.as_array(ctypes.cast(p, DP), shape=(count,)))

    def free(self):
        for p in self.ptrs:
            self.L.hqr_host_free(ctypes.c_void_p(p))
        self.ptrs = []


def measure_e2e(H, torch, L, precision: str, n: int, NB: int, IB: int, steps: int, dist, world: int,
                sample_clocks: bool = False):
    """The same workload through the drop-in C entry points with pinned host arrays:
    Hybrid_tile_QR then Hybrid_make_Q, host<->device copies inside the timed region.
    This region is timed on the host, so by default nvidia-smi does not poll
    during it (sample_clocks: it does, as during the device-timed region)."""
    M = N = n
    L.hqr_set_default_precision(prec_code(H, precision))
    f64 = torch.float64
    gen = torch.empty(M * N, dtype=f64, device="cuda")
    H.check(L.hqr_fill_uniform(M, N, NB, 20151130, gen.data_ptr(), None), "fill")
    torch.cuda.synchronize()
    host = HostArrays(L, torch)
    hA0 = host.empty(M * N)
    hA0.copy_(gen.cpu())
    del gen
    torch.cuda.empty_cache()
    hA = host.empty(M * N)
    hQ = host.empty(M * N)
    hTAU = host.empty((M // 2) * (N // 2))
    hTAU.zero_()
    st = H.status(M, N, NB)
    pa = ctypes.cast(hA.data_ptr(), DP)
    pq = ctypes.cast(hQ.data_ptr(), DP)
    pt = ctypes.cast(hTAU.data_ptr(), DP)
    times, t_qr, t_mq = [], [], []
    ph_qr, ph_mq = [], []   # per call: [h2d, DAG, idle, d2h, device total, host] ms
    ph = (ctypes.c_double * 6)()
    clocks = ClockSampler(torch.cuda.current_device()) if sample_clocks else None
    for it in range(1 + steps):
        if it == 1 and clocks:
            clocks.start()
        hA.copy_(hA0)
        hQ.zero_()
        t0 = time.perf_counter()
        L.Hybrid_tile_QR(ctypes.byref(st), pa, pt, 0, 1, IB)
        H.check(L.hqr_last_error(), "Hybrid_tile_QR")
        t1 = time.perf_counter()
        L.hqr_dropin_phase_ms(ph)
        p_qr = list(ph)
        L.Hybrid_make_Q(ctypes.byref(st), pq, pa, pt, 0, 1, IB)
        H.check(L.hqr_last_error(), "Hybrid_make_Q")
        t2 = time.perf_counter()
        L.hqr_dropin_phase_ms(ph)
        if it > 0:
            ph_qr.append(p_qr)
            ph_mq.append(list(ph))
            times.append(t2 - t0)
            t_qr.append(t1 - t0)
            t_mq.append(t2 - t1)
    clk = clocks.stop() if clocks else "not sampled (host-timed region)"
    L.hqr_set_default_precision(H.HQR_PREC_FP64)
    del hA0, hA, hQ, hTAU
    host.free()
    rate = job_rate(steps * step_flops(M, N), sum(times), dist)
    nbytes = M * N * 8
    tau_b = (M // NB) * (N // NB) * NB * 8
    return {"value": round(rate / 1e12, 6), "unit": "TFLOP/s",
            # Hybrid_tile_QR: A, TAU in and out; Hybrid_make_Q: RY, TAU in (a square
            # Q is written whole on the device, not copied in), Q out (R is the
            # caller's RY with its reflectors zeroed on the host during the DAG)
            "h2d_bytes_per_step": 2 * nbytes + 2 * tau_b,
            "d2h_bytes_per_step": nbytes + tau_b + nbytes,
            "steps": steps, "warmup": 1, "precision": precision,
            "phases_ms": {"Hybrid_tile_QR": round(1e3 * float(np.mean(t_qr)), 3),
                          "Hybrid_make_Q": round(1e3 * float(np.mean(t_mq)), 3)},
            # inside each call, from CUDA events on its stream (means over the steps)
            "device_phases_ms": {
                name: dict(zip(("h2d", "dag", "idle_status", "d2h", "device_total", "host_wall"),
                               (round(float(v), 3) for v in np.mean(np.array(rows), axis=0))))
                for name, rows in (("Hybrid_tile_QR", ph_qr), ("Hybrid_make_Q", ph_mq))},
            "clocks": clk,
            "api": "Hybrid_tile_QR + Hybrid_make_Q (page-locked host arrays from hqr_host_alloc)"}


def lstsq_flops(m: int, n: int, nrhs: int, refine: int, augmented: bool = False) -> float:
    """Algorithmic flops of hqr_lstsq: QR, then per solve Q^T b (4mn - 2n^2 per
    right-hand side) and back substitution (n^2), per refinement step a
    residual (2mn).  hqr_lstsq_aug: the first solve and residual, then per
    step b - A x (2mn), A^T r (2mn), Q^T f and Q [h; d2] (4mn - 2n^2 each)
    and two triangular solves (n^2 each)."""
    per_solve = (4.0 * m * n - 2.0 * n * n + n * n) * nrhs
    if augmented:
        per_step = (2 * 2.0 * m * n + 2 * (4.0 * m * n - 2.0 * n * n) + 2.0 * n * n) * nrhs
        return qr_flops(m, n) + per_solve + 2.0 * m * n * nrhs + refine * per_step
    return qr_flops(m, n) + (refine + 1) * per_solve + refine * 2.0 * m * n * nrhs


def run_lstsq(H, torch, L, args):
    """Least squares min ||A x - b|| through hqr_lstsq (hqr_lstsq_aug with
    --refine-method augmented): A (m x n) = U diag(sigma) V^T with Haar U, V
    and sigma geometric from 1 to 1/kappa, x_true ~ N(0,1), b = A x_true +
    noise N(0,1) (--noise, default 1e-8), nrhs right-hand sides; inputs
    generated with torch on the device, outside the timed region.  Timed:
    whole calls (copy of A, QR, Q^T b, back substitution, refinement).
    Checked against an FP64 least-squares solution of the same problem
    (torch.linalg.lstsq, check only) and against x_true."""
    m, n, nrhs, NB, IB = args.m, args.n, args.nrhs, args.nb, args.ib
    kappa = args.kappa if args.kappa is not None else 1e3
    prec = prec_code(H, args.precision)
    f64 = torch.float64
    gen = torch.Generator(device="cuda")
    gen.manual_seed(20151130)

    def haar(r, c):
        Z = torch.randn(r, c, dtype=f64, device="cuda", generator=gen)
        Q, R = torch.linalg.qr(Z)
        Q *= torch.sign(torch.diagonal(R))
        return Q

    U = haar(m, n)
    U *= kappa ** (-torch.arange(n, dtype=f64, device="cuda") / (n - 1))
    A = U @ haar(n, n).T
    del U
    x_true = torch.randn(n, nrhs, dtype=f64, device="cuda", generator=gen)
    b = A @ x_true + args.noise * torch.randn(m, nrhs, dtype=f64, device="cuda", generator=gen)
    cm = A.T.contiguous()                       # column-major storage of A
    dA = torch.empty(m * n, dtype=f64, device="cuda")
    H.check(L.hqr_colmajor_to_tiles(m, n, NB, cm.data_ptr(), dA.data_ptr(), None), "to tiles")
    del cm
    dB = b.T.contiguous()                       # column-major m x nrhs
    dX = torch.zeros(nrhs, n, dtype=f64, device="cuda")   # column-major n x nrhs
    plan = H.Plan(m, n, NB, IB, prec)
    if args.tree:
        plan.set_tree(args.tree)
    aug = args.refine_method == "augmented"
    torch.cuda.synchronize()
    for _ in range(args.warmup):
        plan.lstsq(dA.data_ptr(), dB.data_ptr(), nrhs, dX.data_ptr(), refine_steps=args.refine, augmented=aug)
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        res = plan.lstsq(dA.data_ptr(), dB.data_ptr(), nrhs, dX.data_ptr(), refine_steps=args.refine,
                         augmented=aug)
    e1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    elapsed = e0.elapsed_time(e1) / 1e3 / args.steps
    plan.close()
    x = dX.T
    x_ref = torch.linalg.lstsq(A, b).solution
    rel = lambda a, r: float(torch.linalg.norm(a - r) / torch.linalg.norm(r))
    flops = lstsq_flops(m, n, nrhs, args.refine, aug)
    line = {
        "metric": "least-squares solve TFLOP/s (QR + Q^T b + back substitution + FP64 refinement)",
        "value": round(flops / elapsed / 1e12, 6), "unit": "TFLOP/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * elapsed, 3),
        "higher_is_better": True, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"least squares, A {m}x{n} = U diag(sigma) V^T (Haar U, V, sigma "
                               f"geometric 1..1/kappa), kappa={kappa:g}, {nrhs} right-hand sides, "
                               f"b = A x_true + {args.noise:g} noise",
                   "m": m, "n": n, "nrhs": nrhs, "kappa": kappa, "NB": NB, "IB": IB,
                   "refine_steps": args.refine, "tree_domain_tiles": args.tree,
                   "refine_method": ("augmented system (hqr_lstsq_aug)" if aug else
                                     "x += R^-1 Q^T (b - A x) (hqr_lstsq)"),
                   "precision": PRECISION_TEXT[args.precision]},
        "accuracy": {"forward_error_vs_fp64_lstsq": rel(x, x_ref),
                     "forward_error_vs_x_true": rel(x, x_true),
                     "fp64_lstsq_error_vs_x_true": rel(x_ref, x_true),
                     "residual_norm_max": max(res),
                     "fp64_lstsq_residual_norm_max": float(torch.linalg.norm(b - A @ x_ref, dim=0).max())},
        "algorithmic_flops": flops,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# batched uneven QR (hqr_batch_*)
# ---------------------------------------------------------------------------
BATCH_METRIC = "batched uneven QR + dormqr TFLOP/s (FP64)"


def batch_shapes(count: int, seed: int):
    """m uniform in {64..2048} step 32, n uniform in {32..m} step 32."""
    rng = np.random.default_rng(seed)
    m = [32 * int(x) for x in rng.integers(2, 65, size=count)]
    n = [32 * int(rng.integers(1, mi // 32 + 1)) for mi in m]
    return m, n


def batch_cpu_sample(m, n, nrhs: int, threads: int, budget_s: float = 15.0):
    """The oracle's restatement of Hybrid_tile_QR + Hybrid_dormqr (NB 32, IB
    32) on matrices of the same workload, one matrix per host thread, until
    about budget_s of wall time.  Returns (flops per second, matrices done)."""
    import concurrent.futures as cf
    import oracle as O
    from hybrid3_gb300 import autotune as AT
    O.set_threads(1)

    def one(b):
        mm, nn = m[b], n[b]
        A = O.to_tiles(O.uniform_matrix(mm, nn, 5000 + b), 32)
        C = O.to_tiles(O.uniform_matrix(mm, 32, 6000 + b), 32)
        t0 = time.perf_counter()
        a, tau = O.tile_qr(A, mm, nn, 32, 32)
        O.dormqr(a, tau, C, mm, nn, 32, 1)
        return time.perf_counter() - t0, AT.qr_flops(mm, nn) + AT.ormqr_flops(mm, nn, nrhs)

    flops, done, t_start = 0.0, 0, time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        b = 0
        while time.perf_counter() - t_start < budget_s and b < len(m):
            futs = [ex.submit(one, i) for i in range(b, min(b + threads, len(m)))]
            b += len(futs)
            for f in futs:
                flops += f.result()[1]
                done += 1
    return flops / (time.perf_counter() - t_start), done


def run_batched_reference(args, rank: int):
    """The reference arm of the batched workload: the reference's algorithm
    (the oracle's restatement of Hybrid_tile_QR + Hybrid_dormqr) on the
    host cores, one matrix per thread, each step a bounded sample (about 10 s)
    of the same shapes.  The reference has no batched mode; this is what
    running its CPU path over the matrices would do."""
    if rank != 0:
        return
    thr = os.cpu_count() or 1
    m, n = batch_shapes(args.batch, 20151130)
    for _ in range(min(args.warmup, 1)):
        batch_cpu_sample(m, n, args.batch_nrhs, thr, 2.0)
    rates, done, walls = [], 0, []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r, k = batch_cpu_sample(m, n, args.batch_nrhs, thr, 10.0)
        walls.append(time.perf_counter() - t0)
        rates.append(r)
        done += k
    value = float(np.mean(rates)) / 1e12
    line = {
        "impl": "reference", "metric": BATCH_METRIC, "value": round(value, 6), "unit": "TFLOP/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * float(np.mean(walls)), 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.batch} independent FP64 matrices (m uniform in {{64..2048}} step 32, "
                               f"n uniform in {{32..m}} step 32), factorization + dormqr on "
                               f"{args.batch_nrhs} right-hand sides; bounded samples of these shapes",
                   "count": args.batch, "nrhs": args.batch_nrhs},
        "cpu_baseline": {"value": round(value, 6), "unit": "TFLOP/s", "cores": thr, "kind": "port",
                         "sample": f"{done} matrices over {args.steps} steps of about 10 s"},
        "e2e": {"value": round(value, 6), "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_batched(H, torch, L, args):
    """4096 independent FP64 QRs of uneven shapes plus dormqr on nrhs
    right-hand sides each, every step two persistent launches over all the
    matrices (hqr_batch_geqrf, hqr_batch_ormqr_t).  NB / IB per size class
    come from the autotuner (timed on samples of the same shapes, outside the
    timed region); matrices are zero-padded to NB multiples and the padding's
    flops are not counted."""
    from hybrid3_gb300 import autotune as AT
    count, nrhs = args.batch, args.batch_nrhs
    m, n = batch_shapes(count, 20151130)
    t0 = time.perf_counter()
    if args.batch_nb:
        nb_ib = tuple(int(x) for x in args.batch_nb.split("/"))
        table = AT.fixed_table(nb_ib[0], nb_ib[1], args.batch_ctas or 1)
    elif args.batch_tune_file and os.path.exists(args.batch_tune_file):
        table = AT.load(args.batch_tune_file)
    else:
        table = AT.tune_batch(H, torch, m, n, nrhs)
        if args.batch_tune_file:
            AT.save(table, args.batch_tune_file)
    tune_s = time.perf_counter() - t0
    pick = [AT.choose(table, a, b, nrhs) for a, b in zip(m, n)]
    nb = [p[0] for p in pick]
    ib = [p[1] for p in pick]
    from collections import Counter
    nb_use = {f"{k[0]}/{k[1]}": v for k, v in sorted(Counter(pick).items())}
    stream = torch.cuda.Stream()
    s = stream.cuda_stream
    d = AT.BatchData(H, torch, m, n, nb, ib, nrhs, 20151130)
    bt = d.batch(H, table["ctas"])
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def step(rec=None):
        with torch.cuda.stream(stream):
            d.restore()
            if rec:
                rec[0].record(stream)
            bt.geqrf(d.pa, d.pt, stream=s, wait=False)
            if rec:
                rec[1].record(stream)
            bt.ormqr_t(d.pa, d.pt, d.pc, nrhs, stream=s, wait=False)
            if rec:
                rec[2].record(stream)

    for _ in range(args.warmup):
        step()
    bt.status(s)
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    recs = [[ev(), ev(), ev()] for _ in range(args.steps)]
    torch.cuda.synchronize()
    t_start, t_end = ev(), ev()
    with torch.cuda.stream(stream):
        t_start.record(stream)
    for r in recs:
        step(r)
    with torch.cuda.stream(stream):
        t_end.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    bt.status(s)
    elapsed = t_start.elapsed_time(t_end) / 1e3 / args.steps
    fact = float(np.mean([r[0].elapsed_time(r[1]) for r in recs])) / 1e3
    appl = float(np.mean([r[1].elapsed_time(r[2]) for r in recs])) / 1e3
    stats = bt.stats(s)   # of the last Q^T C launch
    # per-type task counts and SM time of one more factorization (untimed)
    with torch.cuda.stream(stream):
        d.restore()
    bt.geqrf(d.pa, d.pt, stream=s)
    fstats = bt.stats(s)
    bt.ormqr_t(d.pa, d.pt, d.pc, nrhs, stream=s)   # A and C as after a whole step again
    tot = sum(fstats["cycles"]) or 1
    types = ["geqrt", "tsqrt", "larfb", "ssrfb", "tbuild", "ozprep", "sched"]
    geqrf_tasks = {t: {"count": c, "sm_share": round(y / tot, 4)}
                   for t, c, y in zip(types, fstats["count"], fstats["cycles"]) if c}

    # accuracy on a sample (check only, on the host): R^T R against A^T A, and
    # the least-squares solution R \\ (Q^T c)(1:n) against numpy's FP64 solver
    acc = {"gram_rel_max": 0.0, "lstsq_rel_max": 0.0, "sample": 0}
    f64 = torch.float64
    import scipy.linalg as sla
    for b in (range(0, count, max(1, count // 16)) if not args.no_check else []):
        mm, nn, NB = m[b], n[b], nb[b]
        Mp, Np = d.Mp[b], d.Np[b]
        Cw = -(-nrhs // NB) * NB
        out = {}
        for key, src, cols, off in (("A", d.A, Np, d.a_off), ("A0", d.A0, Np, d.a_off),
                                    ("C", d.C, Cw, d.c_off), ("C0", d.C0, Cw, d.c_off)):
            dst = torch.empty(cols * Mp, dtype=f64, device="cuda")
            H.check(L.hqr_tiles_to_colmajor_padded(Mp, cols, Mp, NB, src.data_ptr() + 8 * int(off[b]),
                                                   dst.data_ptr(), None), "from tiles")
            out[key] = dst.cpu().numpy().reshape(cols, Mp).T
        A0 = out["A0"][:mm, :nn]
        R = np.triu(out["A"][:nn, :nn])
        QtC = out["C"][:nn, :nrhs]
        C0 = out["C0"][:mm, :nrhs]
        G = A0.T @ A0
        acc["gram_rel_max"] = max(acc["gram_rel_max"], float(np.linalg.norm(R.T @ R - G) / np.linalg.norm(G)))
        x = sla.solve_triangular(R, QtC)
        xr = np.linalg.lstsq(A0, C0, rcond=None)[0]
        acc["lstsq_rel_max"] = max(acc["lstsq_rel_max"], float(np.linalg.norm(x - xr) / np.linalg.norm(xr)))
        acc["sample"] += 1

    # end to end: pinned host arrays in, R + reflectors, TAU and Q^T C out.
    # The matrices are cut into P groups of about equal work, each its own
    # batch: group g + 1's inputs are copied in and group g - 1's results out
    # while group g is factored (one stream per direction).
    bt.close()
    e2e = None
    if args.e2e_steps is None or args.e2e_steps > 0:
        ks = args.e2e_steps if args.e2e_steps is not None else args.steps
        P = max(1, min(args.batch_groups, count))
        work = np.cumsum([AT.padded_flops(a, b, k, nrhs) for a, b, k in zip(m, n, nb)])
        cuts = [0] + [int(np.searchsorted(work, work[-1] * (g + 1) / P)) + 1 for g in range(P - 1)] + [count]
        cuts = sorted(set(min(max(c, 0), count) for c in cuts))
        groups = [(cuts[i], cuts[i + 1]) for i in range(len(cuts) - 1) if cuts[i + 1] > cuts[i]]
        bts = [H.Batch(d.Mp[g0:g1], d.Np[g0:g1], nb[g0:g1], ib[g0:g1], max_nrhs=nrhs, ctas_per_sm=table["ctas"])
               for g0, g1 in groups]
        hA0 = torch.empty(d.A0.numel(), dtype=f64).pin_memory()
        hC0 = torch.empty(d.C0.numel(), dtype=f64).pin_memory()
        hA0.copy_(d.A0.cpu())
        hC0.copy_(d.C0.cpu())
        hA = torch.empty_like(hA0).pin_memory()
        hC = torch.empty_like(hC0).pin_memory()
        hT = torch.empty(d.TAU.numel(), dtype=f64).pin_memory()
        s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
        ev_in = [torch.cuda.Event() for _ in groups]
        ev_out = [torch.cuda.Event() for _ in groups]
        rng = lambda o, g0, g1: slice(int(o[g0]), int(o[g1]))
        times = []
        for it in range(1 + ks):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            with torch.cuda.stream(s_in):
                for gi, (g0, g1) in enumerate(groups):
                    a, c = rng(d.a_off, g0, g1), rng(d.c_off, g0, g1)
                    d.A[a].copy_(hA0[a], non_blocking=True)
                    d.C[c].copy_(hC0[c], non_blocking=True)
                    ev_in[gi].record(s_in)
            for gi, (g0, g1) in enumerate(groups):
                stream.wait_event(ev_in[gi])
                bts[gi].geqrf(d.pa[g0:g1], d.pt[g0:g1], stream=s, wait=False)
                bts[gi].ormqr_t(d.pa[g0:g1], d.pt[g0:g1], d.pc[g0:g1], nrhs, stream=s, wait=False)
                ev_out[gi].record(stream)
                with torch.cuda.stream(s_out):
                    s_out.wait_event(ev_out[gi])
                    a, c, t = rng(d.a_off, g0, g1), rng(d.c_off, g0, g1), rng(d.t_off, g0, g1)
                    hA[a].copy_(d.A[a], non_blocking=True)
                    hT[t].copy_(d.TAU[t], non_blocking=True)
                    hC[c].copy_(d.C[c], non_blocking=True)
            torch.cuda.synchronize()
            for b_ in bts:
                b_.status(s)
            if it > 0:
                times.append(time.perf_counter() - t0)
        e2e = {"value": round(d.flops / float(np.mean(times)) / 1e12, 6), "unit": "TFLOP/s",
               "h2d_bytes_per_step": 8 * (d.A0.numel() + d.C0.numel()),
               "d2h_bytes_per_step": 8 * (d.A0.numel() + d.TAU.numel() + d.C0.numel()),
               "steps": ks, "warmup": 1, "groups": len(groups),
               "api": "hqr_batch_geqrf_async + hqr_batch_ormqr_t_async per group, pinned host arrays, "
                      "copies of the next / previous group overlapped on two copy streams"}
        for b_ in bts:
            b_.close()
        del hA0, hC0, hA, hC, hT

    cpu = None
    if not args.no_cpu:
        thr = os.cpu_count() or 1
        v, done = batch_cpu_sample(m, n, nrhs, thr)
        cpu = {"value": round(v / 1e12, 6), "unit": "TFLOP/s", "cores": thr, "kind": "port",
               "sample": f"{done} matrices of the workload (oracle Hybrid_tile_QR + Hybrid_dormqr, NB 32, "
                         f"one matrix per thread)"}
    peak = max(L.hqr_fp64_peak_tflops(None), L.hqr_fp64_mma_peak_tflops(0, None),
               L.hqr_fp64_mma_peak_tflops(1, None))
    value = d.flops / elapsed / 1e12
    padded_flops = sum(AT.qr_flops(a, b) + AT.ormqr_flops(a, b, nrhs) for a, b in zip(d.Mp, d.Np))
    line = {
        "metric": BATCH_METRIC, "value": round(value, 6), "unit": "TFLOP/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * elapsed, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": f"{count} independent FP64 matrices, m uniform in {{64..2048}} step 32, "
                               f"n uniform in {{32..m}} step 32, entries uniform[-1,1) seeded per matrix; "
                               f"factorization + dormqr on {nrhs} right-hand sides each",
                   "count": count, "nrhs": nrhs,
                   "autotune": AT.describe(table), "tune_s": round(tune_s, 2), "nb_ib_use": nb_use,
                   "l2": f"inputs ({8 * d.A0.numel() / 2**30:.1f} GiB) exceed the 129 MB L2; no flush",
                   "parallelism": "one GPU"},
        "phases_ms": {"geqrf": round(1e3 * fact, 3), "ormqr": round(1e3 * appl, 3)},
        "accuracy": acc,
        "roofline": {"kernel": "dag_exec_kernel<fp64, batch>", "bound": "fp64",
                     "achieved": round(d.flops / elapsed / 1e12, 4), "peak": round(peak, 4),
                     "unit": "TFLOP/s", "frac": round(value / peak, 4) if peak > 0 else None,
                     "padded_flops_frac": round(padded_flops / d.flops, 4),
                     "peak_source": "the larger of the FP64 FMA and DMMA issue rates measured in this "
                                    "run (hqr_fp64_peak_tflops, hqr_fp64_mma_peak_tflops)",
                     "traffic": load_batch_traffic(sum(AT.qr_flops(a, b) for a, b in zip(m, n))),
                     "traffic_note": "factorization launch; the 128-matrix capture scaled by flops"},
        "task_counts": {"geqrf": geqrf_tasks, "ormqr": stats["count"]},
        "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": 2 * 3 * args.steps,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=None, help="order (default 16384; 8192 columns with --lstsq)")
    ap.add_argument("--precision", default="split", choices=["split", "fast", "fp32", "fp64"])
    ap.add_argument("--nb", type=int, default=None, help="tile order (default 128 split, 256 fp64)")
    ap.add_argument("--ib", type=int, default=32)
    ap.add_argument("--fp64-nb", type=int, default=256, help="tile order of the plain-FP64 comparison")
    ap.add_argument("--no-compare", action="store_true", help="skip the plain-FP64 comparison run")
    ap.add_argument("--fp64-steps", type=int, default=3, help="timed steps of the plain-FP64 comparison")
    ap.add_argument("--cpu-n", type=int, default=4096, help="CPU sample order")
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--no-check", action="store_true")
    ap.add_argument("--e2e-clocks", action="store_true",
                    help="poll nvidia-smi during the host-timed end-to-end region too")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--kappa", type=float, default=None,
                    help="graded input A = U diag(sigma) V^T with condition number kappa "
                         "(accuracy configuration); default: uniform[-1,1)")
    ap.add_argument("--lstsq", action="store_true",
                    help="least-squares workload through hqr_lstsq instead of QR + make_Q")
    ap.add_argument("--m", type=int, default=32768, help="rows of A for --lstsq")
    ap.add_argument("--nrhs", type=int, default=16, help="right-hand sides for --lstsq")
    ap.add_argument("--refine", type=int, default=1, help="FP64 refinement steps for --lstsq")
    ap.add_argument("--refine-method", default="plain", choices=["plain", "augmented"],
                    help="--lstsq refinement: hqr_lstsq (plain) or hqr_lstsq_aug (augmented system)")
    ap.add_argument("--noise", type=float, default=1e-8,
                    help="--lstsq: b = A x_true + noise N(0,1) (the least-squares residual's size)")
    ap.add_argument("--rows", type=int, default=None,
                    help="rows of A for the QR + make_Q workload (default: square, --n)")
    ap.add_argument("--batched", action="store_true",
                    help="batched uneven QR + dormqr workload through hqr_batch_*")
    ap.add_argument("--batch", type=int, default=4096, help="matrices in the --batched workload")
    ap.add_argument("--batch-nrhs", type=int, default=4, help="right-hand sides per matrix for --batched")
    ap.add_argument("--batch-nb", default=None, help="fixed NB/IB for --batched (default: autotuned)")
    ap.add_argument("--batch-tune-file", default=None,
                    help="autotuner table for --batched: read if it exists, else measured and written")
    ap.add_argument("--batch-groups", type=int, default=4,
                    help="batches the --batched end-to-end run is cut into (copies overlap compute)")
    ap.add_argument("--batch-ctas", type=int, default=0,
                    help="executor CTAs per SM (1 or 2) for --batched with --batch-nb")
    ap.add_argument("--autotune", action="store_true",
                    help="choose precision, NB and IB for the QR + make_Q workload by measuring the "
                         "candidates first (hybrid3_gb300.autotune.tune_single)")
    ap.add_argument("--tree", type=int, default=0,
                    help="domain tree of this many tiles for the TS reduction (0: the flat tree)")
    args = ap.parse_args()
    if args.n is None:
        args.n = 8192 if args.lstsq else 16384
    if args.nb is None:
        args.nb = 128 if args.precision in ("split", "fast", "fp32") else 256

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        # The reference's driver opens two nested parallel regions and only
        # terminates with one thread in the outer one (Hybrid_tile_QR.c:399-405):
        # its build runs with "1,<cores>", set before any OpenMP runtime loads.
        os.environ.setdefault("OMP_NUM_THREADS", f"1,{os.cpu_count() or 1}")
        if args.batched:
            run_batched_reference(args, rank)
        else:
            run_reference(args, rank)
        return

    import torch
    import hybrid3_gb300 as H

    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA device")
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    L = H.lib()
    L.hqr_set_error_mode(H.HQR_ERRORS_RETURN)
    if args.lstsq:
        if rank == 0:
            run_lstsq(H, torch, L, args)
        return
    if args.batched:
        if rank == 0:
            run_batched(H, torch, L, args)
        return
    tuned = None
    if args.autotune:
        # precision, NB and IB for this shape, measured on it (or a scaled
        # sample) before anything is timed; FP64-level precisions only
        from hybrid3_gb300 import autotune as AT
        rows_ = args.rows if args.rows is not None else args.n
        table = AT.tune_single(H, torch, rows_, args.n, want_q=True, reps=1)
        args.precision, args.nb, args.ib = AT.choose_single(table, rows_, args.n)
        e = table["shapes"][0]
        tuned = {"choice": [args.precision, args.nb, args.ib], "sample": e["sample"],
                 "tflops": {f"{p}/{b}/{i}": round(r, 4) for (p, b, i), r in e["rates"].items()}}
    n, NB, IB = args.n, args.nb, args.ib

    # FP64 rates of this GPU: FMA on the CUDA cores and the FP64 tensor cores
    # (DMMA), each an issue-rate probe; the FP64 roofline takes the larger
    fp64_rates = {"ffma": L.hqr_fp64_peak_tflops(None),
                  "dmma_m8n8k4": L.hqr_fp64_mma_peak_tflops(0, None),
                  "dmma_m16n8k16": L.hqr_fp64_mma_peak_tflops(1, None)}
    peak_fp64 = max(fp64_rates.values())
    init = init64 = None
    if args.kappa is not None:
        compare_too = args.precision in ("split", "fast", "fp32") and not args.no_compare
        t = graded_tiles(H, torch, L, n, sorted({NB, args.fp64_nb} if compare_too else {NB}),
                         args.kappa, 1000 + rank)
        init = t[NB]
        init64 = t.get(args.fp64_nb)
    rows = args.rows if args.rows and args.rows != n else None
    M = rows or n
    if rows and args.kappa is not None:
        raise SystemExit("--kappa inputs are square")
    main_run = measure(H, torch, L, args, args.precision, n, NB, IB, args.steps, args.warmup, dist,
                       world, True, not args.no_check, init, rows)
    value = main_run["flops"] / main_run["elapsed"] / 1e12

    e2e = None
    e2e_steps = args.e2e_steps if args.e2e_steps is not None else args.steps
    if e2e_steps > 0 and rows is None:
        e2e = measure_e2e(H, torch, L, args.precision, n, NB, IB, e2e_steps, dist, world, args.e2e_clocks)

    compare = None
    if args.precision in ("split", "fast", "fp32") and not args.no_compare:
        fp = measure(H, torch, L, args, "fp64", n, args.fp64_nb, IB, args.fp64_steps, 1, dist, world, False,
                     not args.no_check, init64, rows)
        fv = fp["flops"] / fp["elapsed"] / 1e12
        compare = {"value": round(fv, 6), "unit": "TFLOP/s", "NB": args.fp64_nb, "IB": IB,
                   "steps": args.fp64_steps, "warmup": 1,
                   "ms_per_step": round(1e3 * fp["elapsed"] / args.fp64_steps, 3),
                   "phases_ms": {"factor": round(1e3 * float(np.mean(fp["fact_s"])), 3),
                                 "make_q": round(1e3 * float(np.mean(fp["mq_s"])), 3)},
                   "fp64_roofline_frac": round(fv / peak_fp64, 4),
                   "accuracy": fp["acc"], "split_over_fp64": round(value / fv, 3)}

    cpu = None
    if rank == 0 and not args.no_cpu:
        t, kind = cpu_sample(args.cpu_n, 256, IB, os.cpu_count() or 1)
        cpu = {"value": round(step_flops(args.cpu_n, args.cpu_n) / t / 1e12, 6), "unit": "TFLOP/s",
               "cores": os.cpu_count() or 1, "kind": kind,
               "sample": f"one {args.cpu_n}x{args.cpu_n} factorization + make_Q (NB=256, IB={IB})"}

    fact_mean = float(np.mean(main_run["fact_s"]))
    achieved = qr_flops(M, n) / fact_mean / 1e12
    peaks = measured_peaks()
    if args.precision in ("split", "fast", "fp32"):
        bf16 = peaks.get("bf16_tflops_sustained") or 1700.0
        prods = split_products(NB) if args.precision == "split" else 10
        peak = bf16 / prods
        roofline = {"kernel": "dag_exec_kernel<split> (factorization launch)", "bound": "tensor",
                    "achieved": round(achieved, 4), "peak": round(peak, 4), "unit": "TFLOP/s",
                    "frac": round(achieved / peak, 4),
                    "peak_source": f"emulated FP64 peak = MEASURED_PEAKS.json bf16_tflops_sustained "
                                   f"({bf16}) / {prods} slice products (of measured)",
                    "traffic": load_traffic(n, NB, "split"),
                    "algorithmic_flops_per_launch": qr_flops(M, n)}
    else:
        roofline = {"kernel": "dag_exec_kernel<fp64> (factorization launch)", "bound": "fp64",
                    "achieved": round(achieved, 4), "peak": round(peak_fp64, 4), "unit": "TFLOP/s",
                    "frac": round(achieved / peak_fp64, 4) if peak_fp64 > 0 else None,
                    "peak_source": "the larger of the FP64 FMA and DMMA issue rates measured in this run "
                                   "(hqr_fp64_peak_tflops, hqr_fp64_mma_peak_tflops); MEASURED_PEAKS.json "
                                   "holds no FP64 figure",
                    "traffic": load_traffic(n, NB, "fp64"),
                    "algorithmic_flops_per_launch": qr_flops(M, n)}
    # this library's kernels per step: factorization (init, seed, executor);
    # make_Q (identity, init, seed, executor, tile transpose, zero reflectors)
    launches_per_step = 3 + 6
    line = {
        "metric": METRIC, "value": round(value, 6), "unit": "TFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * main_run["elapsed"] / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": f"tiled QR + Q generation (make_Q), " +
                               (f"n={n} square" if rows is None else f"{M}x{n} tall") + f", NB={NB}, IB={IB}, " +
                               ("uniform[-1,1) seed 20151130" if args.kappa is None else
                                f"graded A = U diag(sigma) V^T, U, V Haar, kappa={args.kappa:g}"),
                   "n": n, "rows": M, "NB": NB, "IB": IB, "tree_domain_tiles": args.tree,
                   "precision": PRECISION_TEXT[args.precision],
                   "autotuned": tuned,
                   "l2": f"inputs ({8 * M * n / 2**30:.0f} GiB per matrix) exceed the 129 MB L2; no flush",
                   "parallelism": f"replicas x{world}"},
        "phases_ms": {"factor": round(1e3 * fact_mean, 3),
                      "make_q": round(1e3 * float(np.mean(main_run["mq_s"])), 3)},
        "accuracy": main_run["acc"],
        "plain_fp64": compare,
        "roofline": roofline,
        "fp64_peak_measured_tflops": round(peak_fp64, 4),
        "fp64_rates_tflops": {k: round(v, 4) for k, v in fp64_rates.items()},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches_per_step * args.steps,
        "clocks": main_run["clocks"],
        "task_counts_make_q": main_run["stats_mq"]["count"],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
