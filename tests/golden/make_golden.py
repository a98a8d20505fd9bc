"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run in a container that holds the reference sources (zhaijiaqi/AccelES) and the compiled
oracle/_ref library:

    make -C oracle all ref
    python tests/golden/make_golden.py --ref-src /path/to/reference/src

Outputs (small .npz files, committed):
  quantify.npz    quantify_matrix / quantify_vector outputs of
                  src/resources/python/quantify/quantify_util.py:8-49 on seeded inputs
  split.npz       split_approximate (quantify_util.py:173-196) on seeded integer data chosen so
                  that no slice has a tie at its Top-(CK/split) boundary
  gold.npz        spmv_coo_gold_top_k_2 / spmv_coo_gold_top_k / spmv_coo_gold4 / sort_tuples
                  from src/fpga/src/gold_algorithms/gold_algorithms.hpp and
                  src/common/utils/evaluation_utils.hpp, compiled from the reference sources
                  (oracle/_ref/libaes_ref.so)
  xdecode.npz     the x_decoder known-answer case, flag word 0x20080200
                  (src/fpga/src/x_decoder/test_x_decoder.cpp:6), decoded by increment_array
                  (x_decoder.cpp:5-22) as restated bit by bit below
"""
from __future__ import annotations

import argparse
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))


def load_quantify_util(ref_src):
    path = os.path.join(ref_src, "resources", "python", "quantify", "quantify_util.py")
    spec = importlib.util.spec_from_file_location("quantify_util", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def make_quantify(qu, rng):
    out = {}
    cases = []
    # dense sparse-ish matrices like the reference inputs: |N(0,1)| and signed N(0,1)
    for i, (r, c, dens, signed) in enumerate([(64, 50, 0.14, False), (40, 33, 0.3, True),
                                              (25, 64, 0.5, True)]):
        m = rng.standard_normal((r, c)).astype(np.float32)
        if not signed:
            m = np.abs(m)
        m *= (rng.random((r, c)) < dens)
        cases.append(m)
    # exact half-integer boundaries (round-half-to-even) after scaling
    half = np.zeros((4, 31), np.float32)
    for j in range(31):
        half[0, j] = (j + 0.5) / 31.0
        half[1, j] = -(j + 0.5) / 31.0
        half[2, j] = (2 * j + 1) / 62.0
    half[3, 0] = 1.0
    cases.append(half)
    for i, m in enumerate(cases):
        for B in (4, 6, 8):
            for sym in (True, False):
                if not sym and m.min() < 0:
                    continue
                inp = m.astype(np.float64)
                q = qu.quantify_matrix(inp.copy(), B, sym)
                out[f"mat{i}"] = m
                out[f"mat{i}_B{B}_s{int(sym)}"] = np.asarray(q, np.int32)
    # vectors
    vecs = [rng.random(500).astype(np.float32) * 2 - 1, rng.random(1024).astype(np.float32),
            np.abs(rng.standard_normal(300)).astype(np.float32)]
    hv = np.array([(k + 0.5) / 31.0 for k in range(31)] + [1.0], np.float32)
    vecs.append(hv)
    for i, v in enumerate(vecs):
        out[f"vec{i}"] = v
        for B in (4, 6, 8):
            for sym in (True, False):
                if not sym and v.min() < 0:
                    continue
                q = qu.quantify_vector(v.astype(np.float64).copy(), B, sym)
                out[f"vec{i}_B{B}_s{int(sym)}"] = np.asarray(q, np.int32)
    return out


def make_split(qu, rng):
    out = {}
    n_case = 0
    attempt = 0
    while n_case < 3 and attempt < 200:
        attempt += 1
        rows = int(rng.integers(300, 900))
        cols = 64
        split = [32, 8, 1][n_case]
        ck = [128, 64, 50][n_case]
        spm = rng.integers(-31, 32, size=(rows, cols)) * (rng.random((rows, cols)) < 0.3)
        v = rng.integers(-31, 32, size=cols)
        scores = spm @ v
        # reject data with a tie at any slice boundary (numpy's argsort is not stable)
        s = split if split > 1 else 1
        sl = rows // s
        ok = True
        for p in range(s):
            a = p * sl
            b = rows if p == s - 1 else (p + 1) * sl
            seg = np.sort(scores[a:b])[::-1]
            kk = ck // s
            if kk < len(seg) and seg[kk - 1] == seg[kk]:
                ok = False
                break
        if not ok:
            continue
        if split > 1:
            got = qu.split_approximate(spm, v, split, ck)
        else:
            got = qu.top_K_indices(spm @ v, ck)
        out[f"c{n_case}_spm"] = spm.astype(np.int32)
        out[f"c{n_case}_v"] = v.astype(np.int32)
        out[f"c{n_case}_meta"] = np.array([rows, cols, split, ck], np.int64)
        out[f"c{n_case}_idx"] = np.sort(np.asarray(got, np.int64))
        n_case += 1
    return out


def make_gold(rng):
    import oracle as orc
    R = orc.ref_lib()
    if R is None:
        raise SystemExit("oracle/_ref/libaes_ref.so missing: run make -C oracle ref")
    out = {}
    for i, (rows, cols, deg, k, tie) in enumerate([(300, 40, 6, 16, False),
                                                   (500, 30, 4, 64, True),
                                                   (64, 16, 3, 100, True)]):
        r_list, c_list = [], []
        for r in range(rows):
            d = int(rng.integers(1, deg * 2))
            cs = np.sort(rng.choice(cols, size=min(d, cols), replace=False))
            r_list += [r] * len(cs)
            c_list += list(cs)
        row = np.array(r_list, np.uint32)
        col = np.array(c_list, np.uint32)
        if tie:  # few distinct values -> many equal scores, exercises the slot rule
            qv = rng.integers(0, 3, size=row.shape[0]).astype(np.int32)
            vec = rng.integers(0, 3, size=cols).astype(np.int32)
        else:
            qv = rng.integers(-31, 32, size=row.shape[0]).astype(np.int32)
            vec = rng.integers(-31, 32, size=cols).astype(np.int32)
        fv = rng.random(row.shape[0]).astype(np.float32)
        fq = (rng.random(cols) * 2 - 1).astype(np.float32)
        idx, val = orc.gold_topk2(row, col, qv, vec, k, use_ref=True)
        fidx, fval = orc.gold_topk_f32(row, col, fv, fq, k, use_ref=True)
        full = np.zeros(rows, np.float32)
        R.ref_gold4_f32(row.ctypes.data_as(orc._u32p), col.ctypes.data_as(orc._u32p),
                        fv.ctypes.data_as(orc._f32p), row.shape[0], fq.ctypes.data_as(orc._f32p),
                        rows, full.ctypes.data_as(orc._f32p))
        st_idx, st_val = orc.sort_tuples_f32(fidx, fval, use_ref=True)
        for name, a in dict(row=row, col=col, qv=qv, vec=vec, fv=fv, fq=fq, k=np.array([k]),
                            rows=np.array([rows]), topk2_idx=idx, topk2_val=val,
                            topkf_idx=fidx, topkf_val=fval, gold4=full, st_idx=st_idx,
                            st_val=st_val).items():
            out[f"g{i}_{name}"] = a
    return out


def make_xdecode():
    flags = 0x20080200
    P = 30
    x = np.zeros(P, np.int64)
    # increment_array: x[i] += popcount(ptr & ((1 << (i + 1)) - 1)), via the SWAR steps of adder
    for i in range(P):
        c = flags & ((1 << (i + 1)) - 1)
        c = (c & 0x55555555) + ((c & 0xAAAAAAAA) >> 1)
        c = (c & 0x33333333) + ((c & 0xCCCCCCCC) >> 2)
        c = (c & 0x0F0F0F0F) + ((c & 0xF0F0F0F0) >> 4)
        c = (c & 0x00FF00FF) + ((c & 0xFF00FF00) >> 8)
        c = (c & 0x0000FFFF) + ((c & 0xFFFF0000) >> 16)
        x[i] += c
    return {"flags": np.array([flags], np.uint64), "P": np.array([P]), "x": x}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", default="/root/reference/src")
    args = ap.parse_args()
    qu = load_quantify_util(args.ref_src)
    rng = np.random.default_rng(20241203)
    np.savez_compressed(os.path.join(HERE, "quantify.npz"), **make_quantify(qu, rng))
    np.savez_compressed(os.path.join(HERE, "split.npz"), **make_split(qu, rng))
    np.savez_compressed(os.path.join(HERE, "gold.npz"), **make_gold(rng))
    np.savez_compressed(os.path.join(HERE, "xdecode.npz"), **make_xdecode())
    for f in ("quantify.npz", "split.npz", "gold.npz", "xdecode.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")


if __name__ == "__main__":
    main()
