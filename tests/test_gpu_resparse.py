"""ReSparse search on the device: every epoch's metric equals the oracle's for the same seeded
queries (candidates of the pruned matrix by the oracle's two-stage restatement, exact Top-K of
the unpruned FP32 matrix by the oracle's FP32 rescoring of every row)."""
import numpy as np
import pytest

import oracle as orc
from acceles_gb300 import engine as E
from acceles_gb300 import resparse as RS

pytestmark = pytest.mark.gpu


def _fp32_top(ptr, col, val, q, rows, k):
    s = orc.rescore_f32(ptr, col, val, q, np.arange(rows, dtype=np.uint32))
    s = np.where(s == 0, np.float32(0), s)
    return np.lexsort((-np.arange(rows, dtype=np.int64), -s.astype(np.float64)))[:k]


def test_resparse_search_metrics_match_oracle():
    rows, cols, nq, seed = 12000, 256, 6, 5
    ptr, col, val = E.gen_matrix(E.GEN_FIXED_ABSNORMAL, rows, cols, 30, 0, seed=12)
    res = RS.search(ptr, col, val, rows, cols, bits=6, split=32, ck=512, n_queries=nq,
                    seed=seed, max_epochs=4)
    assert [h[1] for h in res["history"][:2]] == [1.0, 0.5]
    rng = np.random.default_rng(seed)
    for epoch, keep, metric, nnz in res["history"]:
        Q = (rng.random((nq, cols)) * 2 - 1).astype(np.float32)
        if keep < 1.0:
            p2, c2, v2 = orc.resparse(ptr, col, val, rows, cols, keep)
        else:
            p2, c2, v2 = ptr, col, val
        assert nnz == len(c2)
        m = orc.Matrix(rows, cols, p2, c2, v2, 6, orc.QUANT_SYM_GLOBAL)
        precs = []
        for q in Q:
            ex = _fp32_top(ptr, col, val, q, rows, 100)
            _, _, cand = m.two_stage(q, 32, 512, 100)
            precs.append(orc.compt_precision(ex, cand))
        assert metric == pytest.approx(orc.convergence_metric(precs), rel=0, abs=1e-12), epoch
