"""GPU: the pre-quantised boundary, the reference's quantised constructor SpMV(q_x, q_y, q_val,
rows, cols, nnz, q_vec) (host_spmv_ucsr.cpp:198-218) and Q_reset(q_type*) (:790), through
aes_create_quantized / aes_set_query_quantized, and Q_read_result's positive filter (:709).

The oracle's quantised COO goes in as given; the candidate set must equal the oracle's Top-CK of
the integer scores, and the streaming Top-K of spmv_coo_gold_top_k_2 (gold_algorithms.hpp:249-308)
on the same integers keeps the same scores (rows tied at its boundary aside)."""
import numpy as np
import pytest

import oracle as orc
from acceles_gb300 import engine as E

pytestmark = pytest.mark.gpu


def quantised_coo(m):
    """COO (row, col, int8 value) of an oracle matrix's quantised CSR."""
    n = np.diff(m.qptr).astype(np.int64)
    row = np.repeat(np.arange(m.rows, dtype=np.uint32), n)
    return row, m.qcol.astype(np.uint32), m.qval.astype(np.int8)


def sorted_candidates(keys, sel):
    """sel in (key desc, row desc) order."""
    sel = np.asarray(sel, np.int64)
    return sel[np.lexsort((-sel, -keys[sel].astype(np.int64)))]


@pytest.mark.parametrize("bits,ck", [(6, 512), (8, 1024), (4, 256)])
def test_quantised_coo_matches_gold_topk2(bits, ck):
    rows, cols, k = 30000, 512, 100
    ptr, col, val = E.gen_matrix(E.GEN_FIXED_ABSNORMAL, rows, cols, 40, 0, seed=31 + bits)
    m = orc.Matrix(rows, cols, ptr, col, val, bits, orc.QUANT_SYM_GLOBAL)
    qrow, qcol, qv = quantised_coo(m)
    eng = E.SpMV(rows, cols, row=qrow, col=qcol, qval=qv, bits=bits, split=1, ck=ck, k_max=k,
                 max_batch=2)
    assert eng.info()["exact_pass"] == 0
    rng = np.random.default_rng(7)
    Q = (rng.random((2, cols)) * 2 - 1).astype(np.float32)  # signed: some scores are negative
    q8 = np.stack([orc.quantize_query(Q[i], bits) for i in range(2)]).astype(np.int8)
    eng.Q_reset_quantized(q8)
    eng(k=k)
    idx, sc = eng.read_topk()
    for i in range(2):
        scores = orc.int_scores(m.qptr, m.qcol, m.qval, rows, q8[i].astype(np.int32))
        keys = orc.cand_keys(scores)
        exp = sorted_candidates(keys, orc.select_split(keys, 1, ck))
        gi, gs, _ = eng.read_candidates(i)
        assert np.array_equal(gi, exp), f"query {i}: candidate set or order differs"
        assert np.array_equal(gs, scores[exp]), f"query {i}: candidate scores differ"
        # the final Top-K ranks the candidates by integer score (no FP32 values given)
        assert np.array_equal(idx[i], exp[:k].astype(np.uint32))
        assert np.array_equal(sc[i], scores[exp[:k]].astype(np.float32))
        # spmv_coo_gold_top_k_2 on the same COO: it keeps non-negative scores only and fills
        # unused slots with (row 0, score 0)
        g_idx, g_val = orc.gold_topk2(qrow, qcol, qv.astype(np.int32), q8[i].astype(np.int32), ck)
        pos = gs > 0
        assert np.array_equal(np.sort(gs[pos]), np.sort(g_val[g_val > 0]))
        t = g_val.min()
        above = set(np.nonzero(scores > t)[0].tolist())
        assert above <= set(g_idx.tolist()) and above <= set(gi.tolist())


def test_positive_filter_as_q_read_result():
    rows, cols, bits, ck = 4000, 256, 6, 512
    ptr, col, val = E.gen_matrix(E.GEN_FIXED_ABSNORMAL, rows, cols, 20, 0, seed=5)
    m = orc.Matrix(rows, cols, ptr, col, val, bits, orc.QUANT_SYM_GLOBAL)
    qrow, qcol, qv = quantised_coo(m)
    rng = np.random.default_rng(3)
    # a query biased negative: the Top-16 of each of the 32 partitions mixes positive and
    # non-positive scores (119 and 393 of the 512 candidates)
    q = (rng.random(cols) - 0.65).astype(np.float32)
    q8 = orc.quantize_query(q, bits).astype(np.int8)
    out = {}
    for flags in (0, E.FLAG_POSITIVE):
        eng = E.SpMV(rows, cols, row=qrow, col=qcol, qval=qv, bits=bits, split=32, ck=ck,
                     k_max=64, flags=flags)
        eng.Q_reset_quantized(q8)
        eng(k=64)
        out[flags] = eng.read_candidates(0)
        eng.close()
    gi, gs, _ = out[0]
    pi, ps, _ = out[E.FLAG_POSITIVE]
    assert np.any(gs <= 0), "the case needs non-positive candidates"
    keep = gs > 0
    assert np.array_equal(pi, gi[keep]) and np.array_equal(ps, gs[keep])
    # sort_tuples order: score descending
    assert np.all(np.diff(ps.astype(np.int64)) <= 0)


def test_quantised_with_fp32_equals_fp32_constructor():
    # values in [0.5, 1): no entry quantises to 0 and no row is left empty, so the quantised COO
    # holds exactly the FP32 entries, and both constructors must give identical results
    rows, cols, bits, ck, k, nq = 40000, 1024, 8, 1024, 100, 3
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, rows, cols, 10, 30, seed=12)
    val = (0.5 + 0.5 * val).astype(np.float32)
    m = orc.Matrix(rows, cols, ptr, col, val, bits, orc.QUANT_SYM_GLOBAL)
    assert np.array_equal(m.qptr, ptr)
    qrow, qcol, qv = quantised_coo(m)
    eng_f = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=bits, split=1, ck=ck, k_max=k,
                   max_batch=nq)
    eng_q = E.SpMV(rows, cols, row=qrow, col=qcol, qval=qv, val=val, bits=bits, split=1, ck=ck,
                   k_max=k, max_batch=nq)
    assert eng_q.info()["exact_pass"] == 1
    Q = np.random.default_rng(9).random((nq, cols)).astype(np.float32)
    eng_f.Q_reset(Q)
    eng_f(k=k)
    fi, fs = eng_f.read_topk()
    eng_q.Q_reset(Q)
    eng_q(k=k)
    qi, qs = eng_q.read_topk()
    assert np.array_equal(fi, qi) and np.array_equal(fs, qs)
    # the same queries given quantised, with their FP32 values for the exact pass
    q8 = np.stack([orc.quantize_query(Q[i], bits) for i in range(nq)]).astype(np.int8)
    eng_q.Q_reset_quantized(q8, Q)
    eng_q(k=k)
    qi2, qs2 = eng_q.read_topk()
    assert np.array_equal(fi, qi2) and np.array_equal(fs, qs2)
    for i in range(nq):
        oi, os_, _ = m.two_stage(Q[i], 1, ck, k)
        assert np.array_equal(qi2[i], oi) and np.array_equal(qs2[i], os_)
    ei, es, _ = eng_q.run_exact(k=k)
    assert ei.shape == (nq, k)


def test_quantised_boundary_errors():
    rows, cols = 1000, 64
    row = np.arange(rows, dtype=np.uint32)
    col = np.zeros(rows, np.uint32)
    qv = np.full(rows, 5, np.int8)
    with pytest.raises(E.AesError) as ex:  # 40 is outside the signed 6-bit range
        E.SpMV(rows, cols, row=row, col=col, qval=np.full(rows, 40, np.int8), bits=6, split=1,
               ck=64, k_max=8)
    assert ex.value.code == E.AES_ERR_INVALID
    with pytest.raises(E.AesError) as ex:
        E.SpMV(rows, cols, row=row, col=col, qval=qv, bits=6, quant=E.QUANT_UNSIGNED_GLOBAL,
               split=1, ck=64, k_max=8)
    assert ex.value.code == E.AES_ERR_UNSUPPORTED
    eng = E.SpMV(rows, cols, row=row, col=col, qval=qv, bits=6, split=1, ck=64, k_max=8)
    with pytest.raises(E.AesError) as ex:
        eng.Q_reset_quantized(np.full(cols, -33, np.int8))
    assert ex.value.code == E.AES_ERR_QUERY
    eng.Q_reset_quantized(np.ones(cols, np.int8))
    eng(k=8)
    with pytest.raises(E.AesError) as ex:  # no FP32 values: no exact pass
        eng.run_exact(k=8)
    assert ex.value.code == E.AES_ERR_STATE
    # every row scores 5 (one entry of value 5 against a query of ones): ties, rows descending
    idx, sc = eng.read_topk()
    assert np.array_equal(idx[0], np.arange(rows - 1, rows - 9, -1, dtype=np.uint32))
    assert np.all(sc[0] == 5.0)
