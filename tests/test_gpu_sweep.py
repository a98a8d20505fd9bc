"""GPU: one variant of the precision sweep (acceles_gb300/sweep.py) on a small matrix, its
recall@K and max relative error against the oracle's float64 Top-K and float64 row scores
computed independently."""
import numpy as np
import pytest

import oracle as orc
from acceles_gb300 import engine as E
from acceles_gb300 import sweep as SW

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bits,quant", [(4, E.QUANT_UNSIGNED_ROW), (6, E.QUANT_SYM_GLOBAL)])
def test_sweep_variant_metrics_match_fp64_oracle(bits, quant):
    rows, cols, nq = 20000, 500, 12
    ptr, col, val = E.gen_matrix(E.GEN_FIXED_ABSNORMAL, rows, cols, 69, 0, seed=3)
    rng = np.random.default_rng(4)
    Q = np.zeros((nq, cols), np.float32)
    for i, r in enumerate(rng.integers(0, rows, nq)):
        Q[i, col[ptr[r]:ptr[r + 1]]] = val[ptr[r]:ptr[r + 1]]
    exact = np.stack([SW.fp64_scores(ptr, col, val, q) for q in Q])
    rec, idx, sc = SW.run_variant(ptr, col, val, rows, cols, Q, exact, bits, quant, 32, 512)
    fi, _ = orc.topk_f64_many(ptr, col, val, rows, cols, Q, max(SW.KS))
    f64 = orc.rows_f64(ptr, col, val, cols, Q, idx)
    for K in SW.KS:
        recall = np.mean([len(set(fi[i, :K].tolist()) & set(idx[i, :K].tolist())) / K
                          for i in range(nq)])
        err = np.max(np.abs(sc[:, :K].astype(np.float64) - f64[:, :K]) / np.abs(f64[:, :K]))
        assert rec["metrics"][K]["recall"] == pytest.approx(recall, abs=1e-12)
        assert rec["metrics"][K]["max_rel_err"] == pytest.approx(err, rel=1e-9, abs=1e-15)
        assert rec["metrics"][K]["max_rel_err"] < 1e-5  # FP32 rescoring of exact rows
