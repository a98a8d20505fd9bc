"""The library-SpMV comparison arm returns the FP32 Top-K: same rows as the path's FP32-only
pass (no near-ties in these seeded inputs), scores within the FP32 summation-order bound."""
import numpy as np
import pytest

from acceles_gb300 import engine as E
from acceles_gb300 import gpu_baseline as G

pytestmark = pytest.mark.gpu


def test_cusparse_topk_matches_exact_pass():
    rows, cols, k = 50000, 1024, 100
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, rows, cols, 10, 30, seed=21)
    Q = np.random.default_rng(3).random((4, cols)).astype(np.float32)
    bi, bs, ms = G.cusparse_topk(ptr, col, val, rows, cols, Q, k)
    assert ms > 0
    eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=8, split=1, ck=1024, k_max=k,
                 max_batch=4)
    eng.Q_reset(Q)
    ei, es, _ = eng.run_exact(k=k)
    for i in range(4):
        assert set(bi[i].tolist()) == set(ei[i].tolist())
        assert np.allclose(bs[i], es[i], rtol=1e-5, atol=0)
