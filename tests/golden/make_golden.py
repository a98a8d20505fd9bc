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
  resparse.npz    resparse_spm (quantify_util.py:375-403) run on seeded dense matrices for
                  several keep ratios; equal |v| never straddle a row's cut (numpy's argsort
                  orders ties differently per platform, so the reference leaves them unspecified)
  mtx/*.mtx +     small Matrix Market files written here, and what the reference's readMtx
  mtx.npz         (src/common/utils/utils.hpp:450-492, compiled in oracle/_ref) returns for them
                  under the argument combinations the reference uses

  python tests/golden/make_golden.py [--only resparse,mtx]
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


RESPARSE_KEEPS = (1.0, 0.9, 0.776, 0.5, 0.05)


def _dense_to_csr(m):
    rows = m.shape[0]
    ptr = np.zeros(rows + 1, np.uint64)
    cols, vals = [], []
    for r in range(rows):
        nz = np.nonzero(m[r])[0]
        cols.extend(nz.tolist())
        vals.extend(m[r, nz].tolist())
        ptr[r + 1] = ptr[r] + len(nz)
    return ptr, np.array(cols, np.uint32), np.array(vals, np.float32)


def make_resparse(qu, rng):
    out = {}
    mats = []
    # continuous values (no ties): |N(0,1)| at 20% density, and signed N(0,1) at 50%
    for (r, c, dens, signed) in [(120, 40, 0.2, False), (60, 30, 0.5, True)]:
        m = rng.standard_normal((r, c)).astype(np.float32)
        if not signed:
            m = np.abs(m)
        m *= (rng.random((r, c)) < dens)
        mats.append(m)
    # repeated magnitudes, one value per row repeated only above the cut: rows of 8 nonzeros
    # whose 3 largest |v| are equal (kept together for every keep >= 0.375) and the rest distinct
    t = np.zeros((20, 24), np.float32)
    for r in range(20):
        cs = rng.choice(24, 8, replace=False)
        v = np.concatenate([np.full(3, 4.0 + r), rng.uniform(0.01, 1.0, 5)]).astype(np.float32)
        v *= rng.choice([-1.0, 1.0], 8).astype(np.float32)
        t[r, cs] = v
    mats.append(t)
    for i, m in enumerate(mats):
        ptr, col, val = _dense_to_csr(m)
        out[f"m{i}_shape"] = np.array(m.shape, np.uint32)
        out[f"m{i}_ptr"], out[f"m{i}_col"], out[f"m{i}_val"] = ptr, col, val
        keeps = RESPARSE_KEEPS if i < 2 else (1.0, 0.776, 0.5, 0.375)
        out[f"m{i}_keeps"] = np.array(keeps)
        for j, keep in enumerate(keeps):
            res = qu.resparse_spm(m.astype(np.float64), keep)
            p2, c2, v2 = _dense_to_csr(res.astype(np.float32))
            out[f"m{i}_k{j}_ptr"], out[f"m{i}_k{j}_col"], out[f"m{i}_k{j}_val"] = p2, c2, v2
    return out


MTX_FILES = {
    "general_1based.mtx": (
        "%%MatrixMarket matrix coordinate real general\n"
        "% a comment line\n"
        "%\n"
        "7 5 10\n"
        "3 2 1.5\n1 1 -2e-3\n7 5 3\n2 4 +4.25\n3 1 0.1\n"
        "1 5 -7.75\n6 3 1e+2\n2 2 0.333333333333\n5 1 -0\n4 4 12\n"),
    "symmetric_1based.mtx": (
        "%%MatrixMarket matrix coordinate real symmetric\n"
        "5 5 7\n"
        "1 1 2.0\n2 1 -1.0\n3 2 0.5\n3 3 4.0\n5 2 1.25\n4 1 -3.5\n5 5 6\n"),
    "pattern_1based.mtx": (
        "%%MatrixMarket matrix coordinate pattern general\n"
        "4 6 5\n"
        "1 6\n4 1\n2 3\n3 3\n1 2\n"),
    "general_0based.mtx": (
        "%%MatrixMarket matrix coordinate real general\n"
        "%\n"
        "6 4 8\n"
        "0 0 1\n5 3 -2.5\n2 1 0.75\n0 3 8\n4 2 -0.125\n1 1 3\n3 0 9.5\n5 0 1e-3\n"),
}
# (file, directed, read_values, zero_indexed, sort) of the reference readMtx; the matching
# library flags are chosen by the test
MTX_CASES = [
    ("general_1based.mtx", 0, 1, 0, 1),
    ("general_1based.mtx", 0, 1, 0, 0),
    ("symmetric_1based.mtx", 0, 1, 0, 0),
    ("symmetric_1based.mtx", 1, 1, 0, 0),
    ("symmetric_1based.mtx", 0, 1, 0, 1),
    ("pattern_1based.mtx", 0, 0, 0, 0),
    ("general_0based.mtx", 0, 1, 1, 0),
]


def make_mtx():
    import oracle as orc
    d = os.path.join(HERE, "mtx")
    os.makedirs(d, exist_ok=True)
    for name, text in MTX_FILES.items():
        with open(os.path.join(d, name), "w") as f:
            f.write(text)
    out = {}
    for i, (name, directed, rv, zero, srt) in enumerate(MTX_CASES):
        rows, cols, r, c, v = orc.ref_read_mtx(os.path.join(d, name), directed, bool(rv),
                                               bool(zero), bool(srt), cap=64)
        out[f"c{i}_args"] = np.array([directed, rv, zero, srt], np.int32)
        out[f"c{i}_name"] = np.array(name)
        out[f"c{i}_shape"] = np.array([rows, cols], np.uint32)
        out[f"c{i}_row"], out[f"c{i}_col"], out[f"c{i}_val"] = r, c, v
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", default=os.environ.get("REF_SRC"), required="REF_SRC" not in os.environ,
                    help="the reference's src directory (or set REF_SRC)")
    ap.add_argument("--only", default="quantify,split,gold,xdecode,resparse,mtx")
    args = ap.parse_args()
    only = set(args.only.split(","))
    qu = load_quantify_util(args.ref_src)
    rng = np.random.default_rng(20241203)
    made = []
    # the first four share one random stream: generate them together or not at all
    if only & {"quantify", "split", "gold", "xdecode"}:
        np.savez_compressed(os.path.join(HERE, "quantify.npz"), **make_quantify(qu, rng))
        np.savez_compressed(os.path.join(HERE, "split.npz"), **make_split(qu, rng))
        np.savez_compressed(os.path.join(HERE, "gold.npz"), **make_gold(rng))
        np.savez_compressed(os.path.join(HERE, "xdecode.npz"), **make_xdecode())
        made += ["quantify.npz", "split.npz", "gold.npz", "xdecode.npz"]
    if "resparse" in only:
        np.savez_compressed(os.path.join(HERE, "resparse.npz"),
                            **make_resparse(qu, np.random.default_rng(375403)))
        made.append("resparse.npz")
    if "mtx" in only:
        np.savez_compressed(os.path.join(HERE, "mtx.npz"), **make_mtx())
        made.append("mtx.npz")
    for f in made:
        print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")


if __name__ == "__main__":
    main()
