#!/usr/bin/env python3
"""Top-100 queries/s of the two-stage low-bit Top-K SpMV on GB300.

Workload: seeded synthetic 10,000,000 x 1024 matrix, row degree uniform in 10..30 (mean 20),
distinct uniform columns, FP32 values U(0,1); 8-bit Ultra-CSR (symmetric global quantiser of the
reference); CK = 1024 candidates, global Top-CK (split 1), K = 100.  Queries: dense U(0,1)^1024.
The reference's matrices are not available; these seeded inputs stand in for them.

A step = one batch of queries through the whole path (quantise, candidate pass, Top-CK select,
FP32 rescoring, Top-K), replayed as a CUDA graph.  `value` is whole-job queries/s with queries
and outputs resident in HBM; `e2e` is the same through the host-buffer C ABI calls
(aes_set_query + aes_run), copies included.  The matrix (about 492 MB of packets + 1.2 GB FP32 CSR) is larger than L2, so every
pass streams from HBM.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Every timed leg runs exactly K steps after W warm-up steps.  The reference arm
(--impl reference) is the reference's CPU method (the oracle port of its gold code) on all host
threads; it builds its own copy of the same seeded matrix through the oracle, so the engine
library is never loaded in that process.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

METRIC = "Top-100 queries/s & HBM GB/s %peak, 10M×1024; batched vs plain, recall=1.0"
ROWS, COLS, DEG_LO, DEG_HI, BITS, CK, K = 10_000_000, 1024, 10, 30, 8, 1024, 100
SEED = 20251203


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_number(name, key):
    """A `key: number` line of a committed ncu summary, if any."""
    p = os.path.join(REPO, "profiles", name)
    if not os.path.exists(p):
        return None
    m = re.search(re.escape(key) + r":\s*([0-9.]+)", open(p).read())
    return float(m.group(1)) if m else None


# kernel sources each committed ncu summary was captured from: a summary whose recorded digest
# differs from the current sources describes an earlier build, and its figures are not reported
PROFILE_SOURCES = {
    "cand_batch_10Mx1024_b8.md": ("aes_batch.cuh", "aes_kernels.cuh"),
    "cand_pass_10Mx1024_b8.md": ("aes_kernels.cuh",),
    "cand_tc_2Mx1024_b4.md": ("aes_tc.cuh", "aes_tc_layout.h", "aes_kernels.cuh"),
}


def source_digest(files):
    h = hashlib.sha256()
    for f in files:
        with open(os.path.join(REPO, "acceles_gb300", "csrc", f), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


def profile_current(name):
    """True when the summary records the digest of the kernel sources built now."""
    p = os.path.join(REPO, "profiles", name)
    if not os.path.exists(p) or name not in PROFILE_SOURCES:
        return False
    m = re.search(r"source_digest:\s*([0-9a-f]{16})", open(p).read())
    return bool(m) and m.group(1) == source_digest(PROFILE_SOURCES[name])


def profile_traffic(name, key="traffic_bytes_per_launch"):
    """DRAM bytes per launch (or per `key`'s unit) of the dominant kernel from the committed ncu
    summary, if it was captured from the current kernel sources."""
    if not profile_current(name):
        return None
    v = profile_number(name, key)
    return int(v) if v is not None else None


def tensor_4bit_leg(local, steps=5, warmup=3):
    """The 4-bit batched sparse-query workload: 20M x 1024, row degree gamma(2, mean 32) capped
    at 512, per-row unsigned 4-bit, 256 queries of 5-30 % density, K 100, CK 256, split 1.  It
    runs the batched candidate pass on the tensor cores (FP8 tcgen05 products of 128-row tiles)
    and, for comparison, with dp4a on the same handle.  Reported: device time of graph-replayed
    steps, the pass's launch time from profiled steps, and whether two queries' Top-K equals the
    FP32-only Top-K of the same engine."""
    from acceles_gb300 import autotune as AT
    from acceles_gb300 import engine as E
    rows, cols, nq, k = 20_000_000, 1024, 256, 100
    ptr, col, val = E.gen_matrix(E.GEN_GAMMA_DEG, rows, cols, 32, 512, seed=4242)
    eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=4, quant=E.QUANT_UNSIGNED_ROW,
                 split=1, ck=256, k_max=k, max_batch=nq, batch_tile=128, sample_stride=256,
                 flags=E.FLAG_GRAPHS | E.FLAG_TENSOR, device=local)
    del ptr, col, val
    Q = AT.sparse_queries(2 * nq, cols, 4244)
    out = {"workload": "20Mx1024 gamma(2, mean 32) cap 512, U(0,1), 4-bit per-row unsigned; "
                       "256 queries of 5-30 % density; K 100, CK 256, split 1",
           "tensor_tiles": eng.info()["tensor_tiles"]}
    for name, tflag in (("tensor_cores", E.FLAG_TENSOR), ("dp4a", 0)):
        eng.retune(flags=E.FLAG_GRAPHS | tflag)
        for s in range(warmup):
            eng.Q_reset(Q[(s % 2) * nq:(s % 2 + 1) * nq])
            eng(k=k)
        ns = 0
        for s in range(steps):
            eng.Q_reset(Q[(s % 2) * nq:(s % 2 + 1) * nq])
            ns += eng(k=k)
        eng.retune(flags=E.FLAG_PROFILE | tflag)
        eng.Q_reset(Q[:nq])
        eng(k=k)
        eng.stats(reset=True)
        eng(k=k)
        st = eng.stats(reset=True)
        # the pass's device time of one step over its blocks of 128 queries (the tensor-core
        # pass launches once per two blocks, on CTA pairs; the dp4a pass once for all blocks)
        out[name] = {"queries_per_s": steps * nq / (ns / 1e9),
                     "ms_per_step": ns / 1e6 / steps,
                     "pass_ms_per_128_queries": st["cand_ms"] / (nq // 128),
                     "pass_launches_timed": int(st["cand_timed"]),
                     "repaired_queries": int(st["repaired"])}
    # dense FP8 products per 128 queries: every 128-row tile times a 128-query operand
    flops = 2.0 * ((rows + 127) // 128) * 128 * 128 * 1024
    tc = out["tensor_cores"]
    tc["dense_tflops"] = flops / (tc["pass_ms_per_128_queries"] / 1e3) / 1e12
    bf16, kind = 1900.0, "fallback"  # TFLOP/s, the fallback when no measured peak file exists
    pk = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(pk) and "bf16_tflops" in json.load(open(pk)):
        bf16, kind = float(json.load(open(pk))["bf16_tflops"]), "measured"
    tc["frac_of_fp8_dense"] = tc["dense_tflops"] / (2 * bf16)
    tc["fp8_dense_peak_note"] = f"FP8 dense taken as twice the {kind} bf16 {bf16:.1f} TFLOP/s"
    eng.retune(flags=E.FLAG_TENSOR)
    eng.Q_reset(Q[:nq])
    eng(k=k)
    idx, _ = eng.read_topk()
    eng.Q_reset(Q[:2])
    ex, _, _ = eng.run_exact(k=k)
    out["top_k_identical_to_fp32_only"] = bool(np.array_equal(idx[:2], ex[:2]))
    eng.close()
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None
        self.th = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.th = threading.Thread(target=self._read, daemon=True)
        self.th.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.th:
            self.th.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def make_matrix(rows=ROWS, oracle_side=False):
    """The seeded 10M x 1024 matrix; oracle_side builds it through the oracle's restatement of
    the same generator (identical arrays), so that the engine library stays unloaded."""
    if oracle_side:
        import oracle as orc
        return orc.gen_matrix(orc.GEN_UNIFORM_DEG, rows, COLS, DEG_LO, DEG_HI, seed=SEED)
    from acceles_gb300 import engine as E
    return E.gen_matrix(E.GEN_UNIFORM_DEG, rows, COLS, DEG_LO, DEG_HI, seed=SEED)


def make_queries(n, seed=SEED + 1):
    return np.random.default_rng(seed).random((n, COLS)).astype(np.float32)


def headline_config(rows, nnz, split, batch):
    """The workload both arms report: identical dicts, so the two lines compare directly."""
    size = f"{rows // 1_000_000}M" if rows >= 1_000_000 else f"{rows // 1000}k"
    return {"workload": f"{size}x1024 deg U{{10..30}} U(0,1), {BITS}-bit Ultra-CSR, "
                        f"CK=1024, K=100, split={split}",
            "rows": rows, "cols": COLS, "nnz": int(nnz), "bits": BITS, "ck": CK,
            "split": split, "k": K, "batch": batch,
            "l2": "inputs larger than L2 (492 MB packets per pass)"}


def cpu_baseline(m, queries, seconds, threads, legs=True):
    """The reference's CPU method (oracle port) on this host: the two-stage method on all
    threads (the reported baseline) and, when `legs`, the two-stage method on one thread and
    the FP32 full Top-K on one and on all threads, each a bounded sample."""
    import oracle as orc
    el, done, _ = orc.bench_two_stage(m, queries, CK, K, nthreads=threads, max_seconds=seconds)
    cb = {"value": done / el, "unit": "queries/s", "cores": threads, "kind": "port",
          "sample": f"{done} queries of the same 10M x 1024 workload: two-stage method "
                    f"(streaming Top-{CK} per row block as gold_algorithms.hpp:249-308, "
                    f"merge, FP32 rescoring, sort_tuples), {threads} threads, {el:.1f} s"}
    if legs:
        short = max(2.0, seconds / 3)
        el1, d1, _ = orc.bench_two_stage(m, queries, CK, K, nthreads=1, max_seconds=short)
        ef, df = orc.bench_fp32_topk(m, queries, K, nthreads=threads, max_seconds=short)
        ef1, df1 = orc.bench_fp32_topk(m, queries, K, nthreads=1, max_seconds=short)
        cb["legs"] = {
            "two_stage_1_thread": {"queries_per_s": d1 / el1, "queries": d1},
            "fp32_full_topk_threads": {"queries_per_s": df / ef, "queries": df, "threads": threads},
            "fp32_full_topk_1_thread": {"queries_per_s": df1 / ef1, "queries": df1},
            "note": "FP32 full Top-K = spmv_coo_gold_top_k (gold_algorithms.hpp:189-247) "
                    "restated; threads = one row block per host thread, merged",
        }
    return cb


def run_reference(args, rank, world):
    """The reference's CPU implementation of the path (the oracle port of its gold code; the
    reference sources are not on the GPU host) on all host threads, same workload, metric and
    config as the GPU arm.  W warm-up steps, then K timed steps; a step is a bounded sample of
    the workload (--cpu-step-queries queries).  Only the oracle library is loaded."""
    if rank != 0:
        return
    import oracle as orc
    threads = os.cpu_count() or 1
    rows = args.rows
    ptr, col, val = make_matrix(rows, oracle_side=True)
    m = orc.Matrix(rows, COLS, ptr, col, val, BITS, orc.QUANT_SYM_GLOBAL)
    per = max(1, args.cpu_step_queries)
    Q = make_queries(per * (args.warmup + args.steps))
    for s in range(args.warmup):
        orc.bench_two_stage(m, Q[s * per:(s + 1) * per], CK, K, nthreads=threads, max_seconds=1e9)
    total, done = 0.0, 0
    for s in range(args.warmup, args.warmup + args.steps):
        el, d, _ = orc.bench_two_stage(m, Q[s * per:(s + 1) * per], CK, K, nthreads=threads,
                                       max_seconds=1e9)
        total += el
        done += d
    qps = done / total
    cb = {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
          "sample": f"{args.steps} steps of {per} queries of the same workload: two-stage "
                    f"method (streaming Top-{CK} per row block as gold_algorithms.hpp:249-308, "
                    f"merge, FP32 rescoring, sort_tuples), {threads} threads, {total:.1f} s"}
    line = {"metric": METRIC, "value": qps, "unit": "queries/s", "impl": "reference",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded; reference matrices not shipped)",
            "config": headline_config(rows, ptr[-1], args.split, args.batch_batched),
            "cpu_baseline": cb,
            "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def check_vs_oracle(m, Q, idx, score, split, nthreads):
    """Every given query against the oracle (bit-exact rows and FP32 scores), against the FP32
    exact Top-K of every row (the reference's FP32 method), and against float64: recall@K of
    each and the largest relative error of a returned FP32 score.  Where the FP32 and float64
    recalls differ, two rows round to the same FP32 score at the K-th place and sort_tuples keeps
    the higher row."""
    import oracle as orc
    oi, os_, on = orc.two_stage_many(m, Q, split, CK, K, nthreads=nthreads)
    exact = True
    for i in range(Q.shape[0]):
        n = int(on[i])
        exact &= bool(np.array_equal(idx[i, :n], oi[i, :n])) and \
            bool(np.array_equal(score[i, :n], os_[i, :n]))
    xi, _ = orc.topk_f32_many(m.ptr, m.col, m.val, m.rows, COLS, Q, K, nthreads=nthreads)
    fi, _ = orc.topk_f64_many(m.ptr, m.col, m.val, m.rows, COLS, Q, K, nthreads=nthreads)
    rec32 = [len(set(xi[i].tolist()) & set(idx[i].tolist())) / K for i in range(Q.shape[0])]
    rec64 = [len(set(fi[i].tolist()) & set(idx[i].tolist())) / K for i in range(Q.shape[0])]
    f64 = orc.rows_f64(m.ptr, m.col, m.val, COLS, Q, idx)
    ok = np.isfinite(f64) & (f64 != 0)
    rel = np.abs(score.astype(np.float64)[ok] - f64[ok]) / np.abs(f64[ok])
    return {"queries": int(Q.shape[0]), "bit_exact_vs_oracle": exact,
            "recall_at_100_vs_fp32_exact_min": min(rec32),
            "recall_at_100_vs_fp64_min": min(rec64),
            "queries_below_1_vs_fp64": int(sum(r < 1.0 for r in rec64)),
            "max_rel_err_vs_fp64": float(rel.max()) if rel.size else 0.0}


SMALL_METRIC = ("Top-100 queries/s, 400k×500 |N(0,1)| 69 nnz/row, 6-bit, SPLIT=32, CK=512 "
                "(plain method, small)")


def run_small(args, rank, world):
    """The reference's small plain-method configuration: 400,000 x 500 at 69 distinct uniform
    columns per row, FP32 values |N(0,1)|, the reference's global 6-bit quantiser, SPLIT=32,
    CK=512, K=100; 100 queries, each a densified random row.  Plain (one candidate pass per
    query) and batched paths on the GPU, every query checked against the oracle, and the
    reference's CPU method on this host's cores."""
    if rank != 0:
        return
    import torch
    import oracle as orc
    from acceles_gb300 import engine as E
    rows, cols, nq, split, ck = 400_000, 500, 100, 32, 512
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    ptr, col, val = E.gen_matrix(E.GEN_FIXED_ABSNORMAL, rows, cols, 69, 0, seed=SEED)
    rng = np.random.default_rng(SEED + 7)
    Q = np.zeros((nq, cols), np.float32)
    for i, r in enumerate(rng.integers(0, rows, nq)):
        Q[i, col[ptr[r]:ptr[r + 1]]] = val[ptr[r]:ptr[r + 1]]
    stream = torch.cuda.Stream()
    dq = torch.from_numpy(Q).cuda()
    di = torch.empty((nq, K), dtype=torch.int32, device="cuda")
    ds = torch.empty((nq, K), dtype=torch.float32, device="cuda")
    out = {}
    for name, bt in (("plain", 1), ("batched", 128)):
        eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=6, quant=E.QUANT_SYM_GLOBAL,
                     split=split, ck=ck, k_max=K, max_batch=nq, batch_tile=bt,
                     flags=E.FLAG_PROFILE)
        run = lambda: eng.run_device(dq.data_ptr(), nq, K, di.data_ptr(), ds.data_ptr(),
                                     stream.cuda_stream)
        for _ in range(args.warmup):
            run()
        torch.cuda.synchronize()
        eng.finish()
        eng.stats(reset=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            run()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        st = eng.stats(reset=True)
        info = eng.info()
        cand_ms = st["cand_ms"] / max(st["cand_timed"], 1)
        out[name] = {"queries_per_s": nq / (ms / 1e3), "ms_per_step": ms,
                     "cand_pass_ms": cand_ms,
                     "cand_pass_gbs": ((info["packets"] * 64 + (info["tiles"] + 1) * 4) / (cand_ms / 1e3) / 1e9
                                       if cand_ms > 0 else None),
                     "repaired": eng.finish() + st["repaired"]}
        # every query against the oracle (outside the timed region)
        eng.Q_reset(Q)
        eng(k=K)
        idx, sc = eng.read_topk()
        m = orc.Matrix(rows, cols, ptr, col, val, 6, orc.QUANT_SYM_GLOBAL)
        exact, rec = True, []
        for i in range(nq):
            oi, os_, _ = m.two_stage(Q[i], split, ck, K)
            exact &= bool(np.array_equal(idx[i, :len(oi)], oi)) and bool(np.array_equal(sc[i, :len(oi)], os_))
            f64 = orc.scores_f64(m.ptr, m.col, m.val, Q[i], rows)
            top = np.argsort(-f64, kind="stable")[:K]
            rec.append(len(set(top.tolist()) & set(idx[i].tolist())) / K)
        out[name]["bit_exact_vs_oracle"] = exact
        out[name]["recall_at_100_vs_fp64_min"] = min(rec)
        eng.close()
    threads = os.cpu_count() or 1
    el, done, _ = orc.bench_two_stage(m, Q, ck, K, nthreads=threads, max_seconds=args.cpu_seconds)
    el1, d1, _ = orc.bench_two_stage(m, Q, ck, K, nthreads=1, max_seconds=max(2.0, args.cpu_seconds / 3))
    line = {"metric": SMALL_METRIC, "value": out["plain"]["queries_per_s"], "unit": "queries/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded; reference matrices not shipped)",
            "config": {"workload": "400kx500 69 nnz/row |N(0,1)|, 6-bit symmetric Ultra-CSR, SPLIT=32, CK=512, K=100, 100 densified-row queries",
                       "rows": rows, "cols": cols, "nnz": int(ptr[-1]), "bits": 6, "split": split,
                       "ck": ck, "k": K, "l2": "packets (about 59 MB) fit in L2"},
            "plain": out["plain"], "batched": out["batched"],
            "cpu_baseline": {"value": done / el, "unit": "queries/s", "cores": threads, "kind": "port",
                             "sample": f"{done} queries: two-stage method, global Top-{ck} "
                                       f"(gold_algorithms.hpp:249-308), FP32 rescoring, {threads} threads, {el:.1f} s",
                             "two_stage_1_thread": d1 / el1}}
    print(json.dumps(line), flush=True)


SERVE_METRIC = ("served queries/s with p50/p99 latency under Poisson arrivals, three resident "
                "matrices (1Mx900 12%, 10Mx1024 deg 20, 20Mx512 gamma mean 32), 8-bit, K in {8,32,100}")


def run_serve(args, rank, world):
    """The serving workload: three device-resident 8-bit matrices, --serve-slots batch slots each
    (the handle and views of it), Poisson arrivals at each offered rate for --serve-seconds, every request
    picking a matrix and K uniformly.  `value` is the served rate at the highest offered rate."""
    if rank != 0:
        return
    import torch
    from acceles_gb300 import engine as E
    from acceles_gb300 import serve as S
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    srv = S.Server(slots=args.serve_slots)
    cols_of, mats = {}, []
    for name, kind, rows, cols, p0, p1, seed in S.serving_specs():
        ptr, col, val = E.gen_matrix(kind, rows, cols, p0, p1, seed=seed)
        info = srv.add_matrix(name, rows, cols, ptr, col, val, max_batch=256, k_max=100, bits=8,
                              split=1, ck=1024, flags=0)
        cols_of[name] = cols
        mats.append({"name": name, "rows": rows, "cols": cols, "nnz": info["nnz"],
                     "slots": info["slots"], "device_bytes": info["device_bytes"]})
        del ptr, col, val
    srv.start()
    names = list(cols_of)
    for w in range(args.warmup):
        S.run_load(srv, names, cols_of, 500, 0.5, seed=90 + w)
    rates = [float(r) for r in args.serve_rates.split(",")]
    legs = []
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    for rate in rates:
        qps, p50, p99, n = S.run_load(srv, names, cols_of, rate, args.serve_seconds, seed=int(rate))
        legs.append({"offered_qps": rate, "served_qps": qps, "p50_ms": p50 * 1e3,
                     "p99_ms": p99 * 1e3, "requests": n})
    clk = clocks.stop()
    in_flight = {m.name: m.max_in_flight for m in srv.mats.values()}
    srv.close()
    top = legs[-1]
    line = {"metric": SERVE_METRIC, "value": top["served_qps"], "unit": "queries/s",
            "n_gpus": 1, "steps": len(legs), "warmup": args.warmup,
            "ms_per_step": args.serve_seconds * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded; reference matrices not shipped)",
            "config": {"workload": "serving: 3 resident matrices, Poisson arrivals, K in {8,32,100}, "
                                   f"8-bit, CK=1024, split=1, max batch 256, {args.serve_slots} batch slots "
                                   "per matrix",
                       "matrices": mats, "offered_rates": rates, "seconds_per_rate": args.serve_seconds},
            "legs": legs, "p50_ms": top["p50_ms"], "p99_ms": top["p99_ms"],
            "max_batches_in_flight_per_matrix": in_flight, "clocks": clk,
            "note": "a step is one offered rate held for seconds_per_rate; latency is submit to "
                    "result on the host, queueing included"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20, help="timed steps of every leg")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=64, help="queries per plain step")
    ap.add_argument("--batch-batched", type=int, default=4096,
                    help="queries per batched step (the headline)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--cpu-step-queries", type=int, default=16,
                    help="queries per step of the reference arm")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-gpu-baseline", action="store_true")
    ap.add_argument("--no-tensor", action="store_true",
                    help="skip the 4-bit tensor-core leg (20M x 1024 sparse-query workload)")
    ap.add_argument("--check", type=int, default=256,
                    help="queries of one batched step checked against the oracle (spread over "
                         "the step); every query of one plain step is checked as well")
    ap.add_argument("--rows", type=int, default=ROWS, help="smaller matrix, for profiling only")
    ap.add_argument("--workload", default="large", choices=["large", "small", "serve"],
                    help="large: 10M x 1024 (the headline); small: the 400k x 500 plain-method "
                         "case; serve: three resident matrices under Poisson arrivals")
    ap.add_argument("--serve-rates", default="1000,10000,50000",
                    help="offered queries/s of the serving workload")
    ap.add_argument("--serve-seconds", type=float, default=4.0)
    ap.add_argument("--serve-slots", type=int, default=2,
                    help="batch slots per matrix (the owning handle and views of it)")
    ap.add_argument("--split", type=int, default=1,
                    help="row partitions with a Top-(CK/split) each (the reference default is 32)")
    ap.add_argument("--bits", type=int, default=8, choices=[4, 6, 8],
                    help="bit width of the large workload (the headline is 8; the reference's "
                         "default is 6)")
    args = ap.parse_args()
    global BITS
    BITS = args.bits
    args.warmup = max(args.warmup, 3)
    args.steps = max(1, args.steps)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "small":
        run_small(args, rank, world)
        return
    if args.workload == "serve":
        run_serve(args, rank, world)
        return

    import torch
    from acceles_gb300 import engine as E

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    rows = args.rows
    ptr, col, val = make_matrix(rows)
    stream = torch.cuda.Stream()  # the engine's kernels and the timing events share it
    sptr = stream.cuda_stream
    threads = os.cpu_count() or 1

    def measure(eng, B, steps, warmup):
        """Device-timed steps of B resident queries; returns (ms, stats, repaired, clocks, pool,
        outputs of one more step on the first B queries of the pool)."""
        npool = B * 4
        Qh = make_queries(npool, seed=SEED + 1 + rank)
        dq = torch.from_numpy(Qh).cuda()
        di = torch.empty((B, K), dtype=torch.int32, device="cuda")
        ds = torch.empty((B, K), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()

        def step(s):
            b = (s % 4) * B
            eng.run_device(dq[b:b + B].data_ptr(), B, K, di.data_ptr(), ds.data_ptr(), sptr)

        for s in range(warmup):
            step(s)
        torch.cuda.synchronize()
        eng.finish()
        eng.stats(reset=True)
        clocks = ClockSampler(local)
        clocks.start()
        time.sleep(0.3)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for s in range(steps):
            step(s)
        e1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        ms = e0.elapsed_time(e1)
        clk = clocks.stop()
        repaired = eng.finish()
        st = eng.stats(reset=True)
        if dist:
            t = torch.tensor([ms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        # one more step on pool slice 0, kept for the oracle check (outside the timed region)
        step(0)
        torch.cuda.synchronize()
        repaired += eng.finish()
        out = (di.cpu().numpy().view(np.uint32).copy(), ds.cpu().numpy().copy())
        return ms, st, repaired, clk, Qh, out

    # The timed steps replay each shape's launches as a CUDA graph (the serving configuration).
    # Per-launch kernel times for the roofline come from a few more steps afterwards with the
    # engine's CUDA-event profiling on, which a graph replay does not record.
    common = dict(bits=BITS, quant=E.QUANT_SYM_GLOBAL, split=args.split, ck=CK, k_max=K, device=local,
                  flags=E.FLAG_GRAPHS)

    def cand_launch_ms(eng, B, n=3):
        """Average candidate-pass launch time (CUDA events on the engine's stream), untimed."""
        eng.retune(flags=E.FLAG_PROFILE)
        Qp = make_queries(B, seed=SEED + 99)
        dq = torch.from_numpy(Qp).cuda()
        di = torch.empty((B, K), dtype=torch.int32, device="cuda")
        ds = torch.empty((B, K), dtype=torch.float32, device="cuda")
        eng.run_device(dq.data_ptr(), B, K, di.data_ptr(), ds.data_ptr(), sptr)
        torch.cuda.synchronize()
        eng.finish()
        eng.stats(reset=True)
        for _ in range(n):
            eng.run_device(dq.data_ptr(), B, K, di.data_ptr(), ds.data_ptr(), sptr)
        torch.cuda.synchronize()
        eng.finish()
        sp = eng.stats(reset=True)
        eng.retune(flags=E.FLAG_GRAPHS)
        return sp["cand_ms"] / max(sp["cand_timed"], 1), sp["cand_launches"] / max(n, 1)

    # plain: one candidate pass per query
    Bp = args.batch
    eng_p = E.SpMV(rows, COLS, ptr=ptr, col=col, val=val, max_batch=Bp, batch_tile=1, **common)
    info = eng_p.info()
    ms_p, st_p, rep_p, clk_p, Qp_pool, out_p = measure(eng_p, Bp, args.steps, args.warmup)
    plain_qps = world * args.steps * Bp / (ms_p / 1e3)
    plain_launch_ms, _ = cand_launch_ms(eng_p, Bp)
    eng_p.close()
    # batched: one candidate pass per 128 queries
    Bb = args.batch_batched
    eng = E.SpMV(rows, COLS, ptr=ptr, col=col, val=val, max_batch=Bb, batch_tile=128, **common)
    ms, st, repaired, clk, Qh, out_b = measure(eng, Bb, args.steps, args.warmup)
    B = Bb
    qps = world * args.steps * Bb / (ms / 1e3)
    batch_launch_ms, cand_per_step = cand_launch_ms(eng, Bb)
    blocks = (Bb + 127) // 128

    # dominant kernel of the batched path: the batched candidate pass; algorithmic bytes of one
    # 128-query block = Ultra-CSR packets + tile row bases + the block's query table
    alg_bytes = info["packets"] * 64 + (info["tiles"] + 1) * 4 + COLS * 128
    cand_ms = batch_launch_ms * cand_per_step / blocks  # device time per 128-query block
    achieved = alg_bytes / (cand_ms / 1e3) / 1e9
    plain_alg = info["packets"] * 64 + (info["tiles"] + 1) * 4 + COLS
    plain_achieved = plain_alg / (plain_launch_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    # the committed ncu summaries are of the 8-bit, one-partition workload at 10M rows
    profiled = BITS == 8 and args.split == 1 and rows == ROWS
    traffic = (profile_traffic("cand_batch_10Mx1024_b8.md", "traffic_bytes_per_block")
               if profiled else None)
    # the batched pass is bound by instruction issue, not HBM: warp instructions per group of
    # four entries (ncu instruction count of the capture) x the groups of one block, over the
    # live time per block at the sampled SM clock; an SM issues at most 4 warp instructions a cycle
    issue = None
    ipg = (profile_number("cand_batch_10Mx1024_b8.md", "warp_instructions_per_group")
           if profiled and profile_current("cand_batch_10Mx1024_b8.md") else None)
    if ipg:
        groups = info["tiles"] * 32 * (511 // (BITS + 11)) // 4
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        mhz = (clk or {}).get("sm_mhz") or (clk or {}).get("sm_max_mhz")
        if mhz:
            ipl = ipg * groups
            ach = ipl / (cand_ms / 1e3 * mhz * 1e6 * sms)
            issue = {"bound": "issue", "unit": "warp instructions per SM cycle", "achieved": ach,
                     "peak": 4.0, "frac": ach / 4.0, "instructions_per_block": ipl,
                     "instructions_per_group": ipg, "groups_per_block": groups,
                     "sm_mhz": mhz, "sms": sms}
    plain_traffic = profile_traffic("cand_pass_10Mx1024_b8.md") if profiled else None

    # end to end through the host-buffer C ABI (batched engine), same K steps
    eng.Q_reset(Qh[:B])
    eng(k=K)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(args.steps):
        b = (s % 4) * B
        eng.Q_reset(Qh[b:b + B])
        eng(k=K)
    e2e_s = time.perf_counter() - t0
    e2e_qps = world * args.steps * B / e2e_s

    # library-SpMV comparison arm on the same matrix and queries (cuSPARSE SpMV + full sort,
    # the reference's GPU baseline method), device time per query
    gpu_lib = None
    if rank == 0 and not args.no_gpu_baseline:
        try:
            from acceles_gb300 import gpu_baseline as G
            _, _, ms_lib = G.cusparse_topk(ptr, col, val, rows, COLS, Qh[:17], K, device=local)
            gpu_lib = {"method": "cuSPARSE SpMV (FP32 CSR) + full descending radix sort + first K",
                       "ms_per_query": ms_lib, "queries_per_s": 1e3 / ms_lib, "queries_timed": 16}
        except Exception as ex:  # report, do not fail the bench
            gpu_lib = {"unavailable": str(ex)[:200]}

    # the FP32-only exact Top-K of the same engine (aes_run_exact: FP32 score of every row, then
    # the Top-K), device time per query; the reference's FP32 method on the GPU
    exact = None
    if rank == 0:
        eng.Q_reset(Qh[:16])
        ei, es, ens = eng.run_exact(k=K)
        exact = {"method": "FP32 score of every row (column-order sums) + Top-K select",
                 "ms_per_query": ens / 1e6 / 16, "queries_per_s": 16 / (ens / 1e9),
                 "queries_timed": 16}
    eng.close()

    # the 4-bit batched sparse-query workload on the tensor cores, beside the dp4a pass
    tensor4 = None
    if rank == 0 and not args.no_tensor:
        try:
            tensor4 = tensor_4bit_leg(local)
        except Exception as ex:  # report, do not fail the bench
            tensor4 = {"unavailable": str(ex)[:200]}

    # correctness of the measured configuration (outside the timed regions): every query of one
    # plain step and a spread of one batched step against the oracle, and against float64
    line_extra = {}
    if rank == 0:
        import oracle as orc
        m = orc.Matrix(rows, COLS, ptr, col, val, BITS, orc.QUANT_SYM_GLOBAL)
        parity = {}
        if args.check > 0:
            sel = np.unique(np.linspace(0, B - 1, min(args.check, B)).astype(np.int64))
            parity["batched"] = check_vs_oracle(m, Qh[sel], out_b[0][sel], out_b[1][sel],
                                                args.split, threads)
            parity["plain"] = check_vs_oracle(m, Qp_pool[:Bp], out_p[0], out_p[1], args.split,
                                              threads)
            if exact is not None:
                allrows = np.arange(rows, dtype=np.uint32)
                s0 = orc.rescore_f32(m.ptr, m.col, m.val, Qh[0], allrows)
                xi, xs = orc.sort_tuples_f32(allrows, s0)
                exact["bit_exact_vs_oracle"] = bool(np.array_equal(ei[0], xi[:K])) and \
                    bool(np.array_equal(es[0], xs[:K]))
        line_extra = {"parity": parity,
                      "parity_checked_queries": sum(v["queries"] for v in parity.values()),
                      "bit_exact_vs_oracle": all(v["bit_exact_vs_oracle"] for v in parity.values())
                      if parity else None,
                      "recall_at_100_vs_fp32_exact": min(v["recall_at_100_vs_fp32_exact_min"]
                                                         for v in parity.values()) if parity else None,
                      "recall_at_100_vs_fp64": min(v["recall_at_100_vs_fp64_min"]
                                                   for v in parity.values()) if parity else None,
                      "max_rel_err_vs_fp64": max(v["max_rel_err_vs_fp64"]
                                                 for v in parity.values()) if parity else None}
        if not args.no_cpu and world == 1:
            Qc = make_queries(max(64, 512), seed=SEED + 5)
            line_extra["cpu_baseline"] = cpu_baseline(m, Qc, args.cpu_seconds, threads)

    if rank == 0:
        line = {
            "metric": METRIC, "value": qps, "unit": "queries/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded; reference matrices not shipped)",
            "config": headline_config(rows, info["nnz"], args.split, Bb),
            "path": "batched (one candidate pass per 128 queries)",
            "plain_leg": {"batch": Bp, "steps": args.steps, "ms_per_step": ms_p / args.steps},
            "parallelism": f"replicas x{world}",
            "batched_qps": qps, "plain_qps": plain_qps, "batched_over_plain": qps / plain_qps,
            "hbm_gbs_batched_pass": achieved, "hbm_gbs_plain_pass": plain_achieved,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": f"k_cand_batch<{BITS},signed,FILTER> (128 queries per matrix read)",
                         "limiter": "CUDA-core integer issue (gathers, byte transposes, dp4a); "
                                    "one matrix read serves 128 queries",
                         "alg_bytes_per_block": alg_bytes, "ms_per_block": cand_ms,
                         "launches_per_step": cand_per_step, "blocks_per_step": blocks,
                         "issue": issue},
            "plain_roofline": {"bound": "hbm", "achieved": plain_achieved, "peak": peak,
                               "unit": "GB/s", "frac": plain_achieved / peak,
                               "traffic": plain_traffic, "kernel": f"k_cand_plain<{BITS},signed,FILTER>",
                               "alg_bytes_per_launch": plain_alg, "launch_ms": plain_launch_ms},
            "e2e": {"value": e2e_qps, "unit": "queries/s", "h2d_bytes_per_step": B * COLS * 4,
                    "d2h_bytes_per_step": B * K * 8},
            "gpu_launches": st["launches"], "repaired_queries": repaired + st["repaired"] + rep_p + st_p["repaired"],
            "clocks": clk, "clocks_plain": clk_p,
            "gpu_library_baseline": gpu_lib,
            "gpu_fp32_exact": exact,
            "tensor_4bit": tensor4,
        }
        line.update(line_extra)
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
