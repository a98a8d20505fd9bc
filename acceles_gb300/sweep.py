"""Precision sweep of the two-stage method on the 400k x 500 matrix (|N(0,1)| values, 69 distinct
uniform columns per row; queries = densified random rows of the matrix).

For each candidate-pass variant (4-bit and 8-bit per-row unsigned quantisation, the reference's
6-bit symmetric quantiser, and the FP32-only single-stage pass) and each CK in {256, 512, 1024},
reports per K in {1, 8, 32, 100}:
  recall@K        |returned Top-K ∩ FP64 exact Top-K| / K, mean over queries
  all_recall@K    fraction of queries with recall@K = 1 (the reference's "recall",
                  quantify_util.py:237-240)
  max_rel_err     max |fp32 score - fp64 score| / |fp64 score| over the returned rows
and the candidate pass's achieved GB/s (Ultra-CSR bytes / device time per launch).

The FP64 reference is computed on the host with numpy (the method's own rescoring precision,
quantify_util.py:354-356).

  python -m acceles_gb300.sweep [--rows 400000] [--queries 100] [--json out.jsonl]
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import engine as E

KS = (1, 8, 32, 100)
CKS = (256, 512, 1024)


def fp64_scores(ptr, col, val, q):
    p = ptr.astype(np.int64)
    prod = val.astype(np.float64) * q.astype(np.float64)[col]
    out = np.zeros(len(p) - 1)
    nz = p[1:] > p[:-1]
    out[nz] = np.add.reduceat(prod, p[:-1][nz])
    return out


def topk_desc(scores, k):
    rows = np.arange(len(scores))
    return np.lexsort((-rows, -scores))[:k]


def metrics(idx, sc, exact, ks):
    out = {}
    for K in ks:
        rec, allr, err = [], [], 0.0
        for i in range(idx.shape[0]):
            ref = set(topk_desc(exact[i], K).tolist())
            got = idx[i, :K]
            hit = len(ref & set(got.tolist())) / K
            rec.append(hit)
            allr.append(1.0 if hit == 1.0 else 0.0)
            e64 = exact[i][got.astype(np.int64)]
            den = np.maximum(np.abs(e64), 1e-30)
            err = max(err, float(np.max(np.abs(sc[i, :K].astype(np.float64) - e64) / den)))
        out[K] = {"recall": float(np.mean(rec)), "all_recall": float(np.mean(allr)),
                  "max_rel_err": err}
    return out


def run_variant(ptr, col, val, rows, cols, Q, exact, bits, quant, split, ck, name=""):
    """One candidate-pass variant at one CK: the engine's Top-max(KS) of every query in Q and its
    metrics against the FP64 scores `exact` [nq, rows], with the candidate pass's GB/s."""
    nq = Q.shape[0]
    eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=bits, quant=quant, split=split,
                 ck=ck, k_max=max(KS), max_batch=nq, batch_tile=1, flags=E.FLAG_PROFILE)
    try:
        info = eng.info()
        eng.Q_reset(Q)
        eng.stats(reset=True)
        eng(k=max(KS))
        st = eng.stats(reset=True)
        idx, sc = eng.read_topk()
    finally:
        eng.close()
    launch_ms = st["cand_ms"] / max(st["cand_timed"], 1)
    gbs = info["packet_bytes"] / (launch_ms / 1e3) / 1e9 if launch_ms > 0 else None
    return {"variant": name, "bits": bits, "ck": ck, "split": split,
            "packet_bytes": info["packet_bytes"], "cand_pass_gbs": gbs,
            "metrics": metrics(idx, sc, exact, KS)}, idx, sc


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--rows", type=int, default=400_000)
    ap.add_argument("--cols", type=int, default=500)
    ap.add_argument("--deg", type=int, default=69)
    ap.add_argument("--queries", type=int, default=100)
    ap.add_argument("--split", type=int, default=32)
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--json", default=None)
    args = ap.parse_args()

    ptr, col, val = E.gen_matrix(E.GEN_FIXED_ABSNORMAL, args.rows, args.cols, args.deg, 0,
                                 seed=args.seed)
    rng = np.random.default_rng(args.seed + 1)
    Q = np.zeros((args.queries, args.cols), np.float32)
    for i, r in enumerate(rng.integers(0, args.rows, args.queries)):
        Q[i, col[ptr[r]:ptr[r + 1]]] = val[ptr[r]:ptr[r + 1]]
    exact = np.stack([fp64_scores(ptr, col, val, q) for q in Q])
    nq = args.queries
    lines = []
    variants = [("B4 per-row unsigned", 4, E.QUANT_UNSIGNED_ROW),
                ("B8 per-row unsigned", 8, E.QUANT_UNSIGNED_ROW),
                ("B6 symmetric (reference default)", 6, E.QUANT_SYM_GLOBAL)]
    for name, bits, quant in variants:
        for ck in CKS:
            rec, _, _ = run_variant(ptr, col, val, args.rows, args.cols, Q, exact, bits, quant,
                                    args.split, ck, name)
            lines.append(rec)
            print(json.dumps(rec), flush=True)
    eng = E.SpMV(args.rows, args.cols, ptr=ptr, col=col, val=val, bits=8, split=1, ck=256,
                 k_max=max(KS), max_batch=nq)
    eng.Q_reset(Q)
    idx, sc, ns = eng.run_exact(k=max(KS))
    fp32_bytes = (args.rows + 1) * 4 + len(col) * 6
    rec = {"variant": "FP32-only plain pass", "bits": 32, "ck": None, "split": 1,
           "bytes": fp32_bytes, "pass_gbs": fp32_bytes / (ns / nq / 1e9) / 1e9,
           "metrics": metrics(idx, sc, exact, KS)}
    lines.append(rec)
    print(json.dumps(rec), flush=True)
    if args.json:
        with open(args.json, "w") as f:
            for l in lines:
                f.write(json.dumps(l) + "\n")


if __name__ == "__main__":
    main()
