"""CPU checks of the precision sweep's metric code (acceles_gb300/sweep.py) on hand-made
inputs: recall@K against the FP64 Top-K (equal scores: the higher row first, the sort_tuples
order the engine returns), the fraction of queries with recall 1, and the largest relative score
error."""
import numpy as np

from acceles_gb300 import sweep as SW


def test_fp64_scores_and_topk_order():
    ptr = np.array([0, 2, 2, 5], np.uint64)
    col = np.array([0, 3, 1, 2, 3], np.uint32)
    val = np.array([1.0, 2.0, 0.5, 0.25, 4.0], np.float32)
    q = np.array([1.0, 2.0, 3.0, 0.5], np.float32)
    s = SW.fp64_scores(ptr, col, val, q)
    assert np.array_equal(s, [1.0 + 1.0, 0.0, 1.0 + 0.75 + 2.0])
    # equal scores: the higher row first
    assert SW.topk_desc(np.array([1.0, 3.0, 3.0, 2.0]), 3).tolist() == [2, 1, 3]


def test_metrics_recall_all_recall_and_error():
    exact = np.array([[5.0, 4.0, 3.0, 2.0, 1.0],
                      [1.0, 2.0, 3.0, 4.0, 5.0]])
    # query 0: its Top-2 exactly, one score off by 1 %; query 1: one of its Top-2 (rows 4, 3)
    idx = np.array([[0, 1], [4, 0]], np.uint32)
    sc = np.array([[5.0, 4.04], [5.0, 1.0]], np.float32)
    m = SW.metrics(idx, sc, exact, (1, 2))
    assert m[1]["recall"] == 1.0 and m[1]["all_recall"] == 1.0
    assert m[2]["recall"] == 0.75 and m[2]["all_recall"] == 0.5
    assert abs(m[2]["max_rel_err"] - 0.01) < 1e-6
    assert m[1]["max_rel_err"] == 0.0
