"""ReSparse: per-row pruning of the matrix before quantisation, and the search for the
smallest keep ratio whose candidate precision stays within a factor of the unpruned one.

The pruning itself is the library's host pass (aes_resparse; resparse_spm,
quantify_util.py:375-403).  The search follows the bisection of
search_best_resparse_ratio.py:55-117:

  epoch 0 measures the unpruned matrix (keep 1.0) and sets the bar to its metric x threshold;
  epoch 1 tries keep 0.5; after every later measurement the bound on the passing side moves to
  the tried ratio and the next ratio is the midpoint rounded to 3 decimals; the search stops
  when that midpoint was tried before and answers the upper bound.

The metric of an epoch (print_convergence_matrics, quantify_util.py:413-437) is the weighted
sum over K in {1, 8, 16, 32, 50, 75, 100} (weights 1/K, K=1 weighted 1) of the mean
precision |candidates ∩ exact Top-K| / K (compt_precision, :198-219) over the epoch's queries.
Here every epoch draws fresh seeded dense queries U(-1, 1)^cols (create_v, :137-144), the
candidates come from a device handle built on the pruned matrix, and the exact Top-K from
the FP32-only pass over the unpruned matrix on the device (the reference uses numpy's FP64
product; the two orders differ only where FP32 rounding reorders near-equal scores).
"""
from __future__ import annotations

import numpy as np

from . import engine as E

TOP_KS = (1, 8, 16, 32, 50, 75, 100)
_WEIGHTS = tuple(1.0 / k for k in TOP_KS)


def precision_at(exact_top, cand):
    """Fraction of exact_top[:K] found among the candidates, for each K of TOP_KS."""
    c = set(np.asarray(cand, np.int64).tolist())
    ex = np.asarray(exact_top, np.int64)
    return [sum(1 for x in ex[:k].tolist() if x in c) / k for k in TOP_KS]


def epoch_metric(precisions):
    """Weighted sum of the per-K mean precisions of one epoch."""
    p = np.asarray(precisions, np.float64)
    means = [float(sum(p[:, i]) / len(p)) for i in range(len(TOP_KS))]
    return sum(m * w for m, w in zip(means, _WEIGHTS))


def bisect_keep(evaluate, accuracy_threshold=0.999, max_epochs=100):
    """Bisection over keep ratios with evaluate(keep, epoch) -> metric.

    Returns (keep ratio, history of (epoch, keep, metric)); keep is None if max_epochs pass
    without convergence."""
    history = []
    lo, hi = 0.0, 1.0
    tried = set()
    bar = None
    keep = 1.0
    for epoch in range(max_epochs):
        if epoch == 1:
            keep = (lo + hi) / 2
        metric = evaluate(keep, epoch)
        tried.add(keep)
        history.append((epoch, keep, metric))
        if bar is None:
            bar = metric * accuracy_threshold
            continue
        if metric >= bar:
            hi = keep
        else:
            lo = keep
        keep = round((lo + hi) / 2, 3)
        if keep in tried:
            return hi, history
    return None, history


def search(ptr, col, val, rows, cols, bits=6, quant=E.QUANT_SYM_GLOBAL, split=32, ck=512,
           k=100, n_queries=100, accuracy_threshold=0.999, seed=0, device=0, max_epochs=100,
           log=None):
    """Smallest ReSparse keep ratio of a sorted CSR; see the module docstring.

    Returns {"keep", "history": [(epoch, keep, metric, nnz)], "nnz"}."""
    k = min(k, max(TOP_KS))
    rng = np.random.default_rng(seed)
    full = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=bits, quant=quant, split=split,
                  ck=ck, k_max=max(TOP_KS), max_batch=n_queries, device=device)
    nnz_of = {}

    def evaluate(keep, epoch):
        Q = (rng.random((n_queries, cols)) * 2 - 1).astype(np.float32)
        full.Q_reset(Q)
        exact, _, _ = full.run_exact(k=max(TOP_KS))
        if keep >= 1.0:
            eng, nnz = full, len(col)
        else:
            p2, c2, v2 = E.resparse(ptr, col, val, rows, cols, keep)
            nnz = len(c2)
            eng = E.SpMV(rows, cols, ptr=p2, col=c2, val=v2, bits=bits, quant=quant,
                         split=split, ck=ck, k_max=max(TOP_KS), max_batch=n_queries,
                         device=device)
        eng.Q_reset(Q)
        eng(k=max(TOP_KS))
        prec = [precision_at(exact[i], eng.read_candidates(i)[0]) for i in range(n_queries)]
        if eng is not full:
            eng.close()
        m = epoch_metric(prec)
        nnz_of[keep] = nnz
        if log:
            log({"epoch": epoch, "keep": keep, "metric": m, "nnz": nnz})
        return m

    try:
        keep, hist = bisect_keep(evaluate, accuracy_threshold, max_epochs)
    finally:
        full.close()
    return {"keep": keep, "history": [(e, r, m, nnz_of[r]) for e, r, m in hist],
            "nnz": len(col)}


def _normal_rows(rows, cols, deg_lo, deg_hi, seed):
    """Seeded CSR like the reference's synthetic matrices (create_matrices.py:57-137): degree
    uniform in [deg_lo, deg_hi], uniform columns (distinct here), N(0,1) values scaled to unit
    L2 norm per row."""
    ptr, col, _ = E.gen_matrix(E.GEN_UNIFORM_DEG, rows, cols, deg_lo, deg_hi, seed=seed)
    rng = np.random.default_rng(seed + 1)
    val = rng.standard_normal(len(col))
    deg = np.diff(ptr).astype(np.int64)
    rid = np.repeat(np.arange(rows), deg)
    norm = np.sqrt(np.bincount(rid, weights=val * val, minlength=rows))
    val = (val / norm[rid]).astype(np.float32)
    return ptr, col, val


def main():
    import argparse
    import json
    import time
    ap = argparse.ArgumentParser(description="ReSparse keep-ratio search on the device")
    ap.add_argument("--rows", type=int, default=5_000_000)
    ap.add_argument("--cols", type=int, default=1024)
    ap.add_argument("--deg-lo", type=int, default=10)
    ap.add_argument("--deg-hi", type=int, default=30)
    ap.add_argument("--mtx", default=None, help="read this Matrix Market file instead")
    ap.add_argument("--zero-indexed", action="store_true")
    ap.add_argument("--bits", type=int, default=6)
    ap.add_argument("--split", type=int, default=32)
    ap.add_argument("--ck", type=int, default=512)
    ap.add_argument("--queries", type=int, default=100)
    ap.add_argument("--threshold", type=float, default=0.9999)
    ap.add_argument("--seed", type=int, default=7)
    args = ap.parse_args()
    t0 = time.perf_counter()
    if args.mtx:
        rows, cols, r, c, v = E.read_mtx(args.mtx, E.MTX_SORT | (E.MTX_ZERO_INDEXED if args.zero_indexed else 0))
        ptr = np.zeros(rows + 1, np.uint64)
        np.add.at(ptr, r.astype(np.int64) + 1, 1)
        ptr = np.cumsum(ptr).astype(np.uint64)
        col, val = c, v
        src = args.mtx
    else:
        rows, cols = args.rows, args.cols
        ptr, col, val = _normal_rows(rows, cols, args.deg_lo, args.deg_hi, args.seed)
        src = (f"{rows}x{cols} seeded, degree U{{{args.deg_lo}..{args.deg_hi}}}, "
               "N(0,1) values with unit row norm")
    print(json.dumps({"matrix": src, "nnz": int(len(col)), "load_s": time.perf_counter() - t0}),
          flush=True)
    t0 = time.perf_counter()
    res = search(ptr, col, val, rows, cols, bits=args.bits, split=args.split, ck=args.ck,
                 n_queries=args.queries, accuracy_threshold=args.threshold, seed=args.seed,
                 log=lambda d: print(json.dumps(d), flush=True))
    keep = res["keep"]
    nnz_keep = dict((r, n) for _, r, _, n in res["history"]).get(keep)
    print(json.dumps({"converged_keep": keep, "nnz_before": res["nnz"], "nnz_after": nnz_keep,
                      "epochs": len(res["history"]), "search_s": time.perf_counter() - t0,
                      "bits": args.bits, "split": args.split, "ck": args.ck,
                      "threshold": args.threshold, "queries_per_epoch": args.queries}),
          flush=True)


if __name__ == "__main__":
    main()
