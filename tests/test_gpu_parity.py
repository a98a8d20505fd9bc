"""GPU parity: the sm_103a path through the C ABI against the CPU oracle on the same seeded
inputs.  Integer candidate keys and Top-K row indices must be bit-exact; FP32 exact-pass
scores are compared bit for bit (both sides compute separately rounded multiply-then-add in
column order), with the 1e-5 relative bound of the method as the stated tolerance."""
import numpy as np
import pytest

import oracle as orc
from acceles_gb300 import engine as E

pytestmark = pytest.mark.gpu

RTOL = 1e-5  # exact-pass tolerance against the FP32 oracle


def make(rows, cols, kind, p0, p1, seed, bits, quant, split, ck, k, nq=1, **kw):
    ptr, col, val = E.gen_matrix(kind, rows, cols, p0, p1, seed=seed)
    m = orc.Matrix(rows, cols, ptr, col, val, bits, quant)
    eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=bits, quant=quant, split=split,
                 ck=ck, k_max=k, max_batch=nq, **kw)
    return m, eng


def queries(cols, nq, seed, signed=False):
    rng = np.random.default_rng(seed)
    q = rng.random((nq, cols)).astype(np.float32)
    if signed:
        q = q * 2 - 1
    return q


def check_run(m, eng, Q, split, ck, k):
    eng.Q_reset(Q)
    eng(k=k)
    idx, sc = eng.read_topk()
    for i in range(Q.shape[0]):
        oi, os_, cand = m.two_stage(Q[i], split, ck, k)
        n = len(oi)
        assert np.array_equal(idx[i, :n], oi), f"query {i}: Top-K rows differ"
        assert np.allclose(sc[i, :n], os_, rtol=RTOL, atol=0), f"query {i}: scores"
        assert np.array_equal(sc[i, :n], os_), f"query {i}: scores not bit-identical"
        assert np.all(idx[i, n:] == 0xFFFFFFFF)
        # candidate set and its (key desc, row desc) order
        gi, _, gk = eng.read_candidates(i)
        keys = m.keys(Q[i])
        exp = cand[np.lexsort((-cand.astype(np.int64), -keys[cand].astype(np.int64)))]
        assert np.array_equal(gi, exp), f"query {i}: candidate set differs"


@pytest.mark.parametrize("bits", [4, 6, 8])
@pytest.mark.parametrize("quant", [0, 1, 2])
def test_candidate_keys_bit_exact(bits, quant):
    rows, cols = 6000, 1024
    m, eng = make(rows, cols, E.GEN_UNIFORM_DEG, 10, 30, 100 + bits, bits, quant, 1, 256, 16)
    for s in range(2):
        q = queries(cols, 1, s, signed=(quant == 0))[0]
        got = eng.score_all(q)
        assert np.array_equal(got, m.keys(q))


@pytest.mark.parametrize("bits,quant,split,ck", [(8, 0, 1, 1024), (6, 0, 32, 512),
                                                 (4, 1, 1, 256), (8, 2, 8, 512),
                                                 (6, 1, 32, 1024)])
def test_two_stage_matches_oracle(bits, quant, split, ck):
    rows, cols, k = 20000, 1024, 100
    m, eng = make(rows, cols, E.GEN_UNIFORM_DEG, 10, 30, 7, bits, quant, split, ck, k, nq=3)
    check_run(m, eng, queries(cols, 3, 1, signed=(quant == 0)), split, ck, k)


@pytest.mark.parametrize("split,ck,nq,bt", [(32, 1024, 3, 1), (32, 1024, 40, 128),
                                            (2000, 4000, 3, 1), (600, 1200, 20, 128)])
def test_partition_bounds_per_tile(split, ck, nq, bt):
    """Integer keys with many row partitions: the candidate passes compare each row with the
    lowest threshold of the partitions its tile touches and check a hit against its own
    partition.  Short slices make tiles straddle several partitions; 600 and 2000 partitions
    keep their thresholds in global memory."""
    rows, cols, k = 20000, 1024, 100
    m, eng = make(rows, cols, E.GEN_UNIFORM_DEG, 10, 30, 31, 8, 0, split, ck, k, nq=nq,
                  batch_tile=bt)
    check_run(m, eng, queries(cols, nq, 5, signed=True), split, ck, k)


def test_config1_shape_absnormal_b6_split32():
    # 400k x 500 at 69 nnz/row in the reference, here scaled down; queries = densified rows
    rows, cols = 12800, 500
    m, eng = make(rows, cols, E.GEN_FIXED_ABSNORMAL, 69, 0, 3, 6, 0, 32, 512, 100, nq=4)
    rng = np.random.default_rng(9)
    Q = np.zeros((4, cols), np.float32)
    for i, r in enumerate(rng.integers(0, rows, 4)):
        Q[i, m.col[m.ptr[r]:m.ptr[r + 1]]] = m.val[m.ptr[r]:m.ptr[r + 1]]
    check_run(m, eng, Q, 32, 512, 100)


def test_long_rows_span_tiles_gamma():
    rows, cols = 3000, 1024
    m, eng = make(rows, cols, E.GEN_GAMMA_DEG, 200, 1024, 4, 8, 0, 1, 512, 64, nq=2)
    check_run(m, eng, queries(cols, 2, 5, signed=True), 1, 512, 64)


@pytest.mark.parametrize("rows", [1, 5, 33, 100])
def test_tiny_matrices_and_ragged_partitions(rows):
    cols = 64
    m, eng = make(rows, cols, E.GEN_UNIFORM_DEG, 1, 8, rows, 6, 0, 32, 64, 10, nq=2)
    check_run(m, eng, queries(cols, 2, rows, signed=True), 32, 64, 10)


def test_k_larger_than_candidates():
    rows, cols = 50, 128
    m, eng = make(rows, cols, E.GEN_UNIFORM_DEG, 3, 9, 2, 8, 0, 1, 64, 100)
    check_run(m, eng, queries(cols, 1, 3), 1, 64, 100)


def test_repair_path_threshold_miss():
    """Scores decreasing with the row index put the global top rows in the first (sampled)
    tile, so the sample threshold admits too few rows; the exact slow path repairs the query."""
    rows, cols = 40000, 256
    ptr = np.arange(rows + 1, dtype=np.uint64) * 4
    col = np.tile(np.array([0, 1, 2, 3], np.uint32), rows)
    val = np.repeat(np.linspace(1.0, 0.01, rows).astype(np.float32), 4)
    m = orc.Matrix(rows, cols, ptr, col, val, 8, 0)
    eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=8, quant=0, split=1, ck=512,
                 k_max=100, sample_stride=4)
    q = np.ones((1, cols), np.float32)
    check_run(m, eng, q, 1, 512, 100)


def test_zero_query_all_ties():
    rows, cols = 5000, 1024
    m, eng = make(rows, cols, E.GEN_UNIFORM_DEG, 10, 30, 8, 8, 0, 1, 512, 100)
    check_run(m, eng, np.zeros((1, cols), np.float32), 1, 512, 100)


def test_batch_equals_single_queries():
    rows, cols = 20000, 1024
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, rows, cols, 10, 30, seed=21)
    Q = queries(cols, 5, 2)
    eb = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=8, split=1, ck=1024, k_max=100,
                max_batch=5)
    eb.Q_reset(Q)
    eb(k=100)
    bi, bs = eb.read_topk()
    es = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=8, split=1, ck=1024, k_max=100)
    for i in range(5):
        es.Q_reset(Q[i])
        es(k=100)
        si, ss = es.read_topk()
        assert np.array_equal(si[0], bi[i]) and np.array_equal(ss[0], bs[i])


def test_run_device_path():
    import torch
    rows, cols = 20000, 1000
    m, eng = make(rows, cols, E.GEN_UNIFORM_DEG, 10, 30, 31, 8, 0, 1, 1024, 100, nq=4)
    Q = queries(cols, 4, 6)
    dq = torch.from_numpy(Q).cuda()
    di = torch.empty((4, 100), dtype=torch.int32, device="cuda")
    ds = torch.empty((4, 100), dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream()
    eng.run_device(dq.data_ptr(), 4, 100, di.data_ptr(), ds.data_ptr(), s.cuda_stream)
    assert eng.finish() == 0
    gi = di.cpu().numpy().view(np.uint32)
    gs = ds.cpu().numpy()
    for i in range(4):
        oi, os_, _ = m.two_stage(Q[i], 1, 1024, 100)
        assert np.array_equal(gi[i, :len(oi)], oi) and np.array_equal(gs[i, :len(oi)], os_)


def test_unsigned_query_rejected():
    rows, cols = 1000, 64
    m, eng = make(rows, cols, E.GEN_UNIFORM_DEG, 2, 6, 1, 8, 1, 1, 64, 10)
    eng.Q_reset(-np.ones(cols, np.float32))
    with pytest.raises(E.AesError) as ei:
        eng(k=10)
    assert ei.value.code == E.AES_ERR_QUERY


def test_trunc_query_quantiser():
    rows, cols = 5000, 300
    m, eng = make(rows, cols, E.GEN_FIXED_ABSNORMAL, 40, 0, 12, 6, 0, 1, 256, 50,
                  query_quant=E.QQ_TRUNC)
    q = queries(cols, 1, 4, signed=True)[0]
    assert np.array_equal(eng.score_all(q), m.keys(q, qq=orc.QQ_TRUNC))


def test_reference_api_shape():
    """Q_reset / operator() / Q_read_result in the reference's calling order (main,
    host_spmv_ucsr.cpp:1084-1113)."""
    rows, cols = 8000, 512
    m, eng = make(rows, cols, E.GEN_UNIFORM_DEG, 10, 30, 40, 6, 0, 32, 512, 100)
    q = queries(cols, 1, 41, signed=True)[0]
    eng.Q_reset(q, 0)
    ns = eng(True, 0)
    assert ns > 0
    res, idx = [], []
    eng.Q_read_result(res, idx, 0)
    keys = m.keys(q)
    assert len(idx) == len(res) == 512
    assert all(keys[i] ^ 0x80000000 == (s & 0xFFFFFFFF) for i, s in zip(idx, res))
    order = list(zip(res, idx))
    assert order == sorted(order, reverse=True)


# ---- batched candidate pass (one matrix read per tile of up to 128 queries) -------------------

@pytest.mark.parametrize("bits,quant,split,ck,nq", [(8, 0, 1, 1024, 128), (6, 0, 32, 512, 37),
                                                   (4, 1, 1, 256, 200), (8, 2, 8, 512, 64),
                                                   (4, 0, 32, 1024, 130)])
def test_batched_matches_oracle(bits, quant, split, ck, nq):
    rows, cols, k = 20000, 1024, 100
    m, eng = make(rows, cols, E.GEN_UNIFORM_DEG, 10, 30, 17 + bits, bits, quant, split, ck, k,
                  nq=nq, batch_tile=128)
    assert eng.info()["batch_tile"] == 128
    Q = queries(cols, nq, 11, signed=(quant == 0))
    eng.Q_reset(Q)
    eng(k=k)
    idx, sc = eng.read_topk()
    for i in range(0, nq, max(1, nq // 9)):
        oi, os_, cand = m.two_stage(Q[i], split, ck, k)
        n = len(oi)
        assert np.array_equal(idx[i, :n], oi), i
        assert np.array_equal(sc[i, :n], os_), i
        gi, _, _ = eng.read_candidates(i)
        keys = m.keys(Q[i])
        exp = cand[np.lexsort((-cand.astype(np.int64), -keys[cand].astype(np.int64)))]
        assert np.array_equal(gi, exp), i


@pytest.mark.parametrize("bits,lo,hi", [(8, 1, 5), (8, 3, 14), (8, 9, 11), (4, 2, 9),
                                         (6, 1, 3)])
def test_batched_short_rows(bits, lo, hi):
    """Rows of a few entries: a tile whose rows, each padded to a multiple of four entries, no
    longer fit the per-warp records keeps the unpadded walk, so one pass mixes both layouts."""
    rows, cols, k, nq = 30000, 512, 50, 130
    m, eng = make(rows, cols, E.GEN_UNIFORM_DEG, lo, hi, 40 + lo, bits, 0, 4, 256, k, nq=nq,
                  batch_tile=128)
    Q = queries(cols, nq, 19, signed=True)
    eng.Q_reset(Q)
    eng(k=k)
    idx, sc = eng.read_topk()
    for i in range(0, nq, 11):
        oi, os_, cand = m.two_stage(Q[i], 4, 256, k)
        n = len(oi)
        assert np.array_equal(idx[i, :n], oi), i
        assert np.array_equal(sc[i, :n], os_), i
        gi, _, _ = eng.read_candidates(i)
        keys = m.keys(Q[i])
        exp = cand[np.lexsort((-cand.astype(np.int64), -keys[cand].astype(np.int64)))]
        assert np.array_equal(gi, exp), i


@pytest.mark.parametrize("warps", [1, 3, 8, 12])
def test_batched_warps_per_cta(warps):
    """Fewer warps per CTA than fit (aes_params.batch_warps) give the same results: the tiles a
    CTA takes, and so the ranges its warps walk, change with the warp count."""
    rows, cols, k, nq = 25000, 1024, 100, 130
    m, eng = make(rows, cols, E.GEN_UNIFORM_DEG, 10, 30, 5 + warps, 8, 0, 1, 512, k, nq=nq,
                  batch_tile=128)
    Q = queries(cols, nq, 23, signed=True)
    eng.Q_reset(Q)
    eng(k=k)
    ref = tuple(x.copy() for x in eng.read_topk())
    assert eng.info()["batch_warps"] == 16
    eng.retune(batch_warps=warps)
    assert eng.info()["batch_warps"] == warps
    eng.Q_reset(Q)
    eng(k=k)
    idx, sc = eng.read_topk()
    assert np.array_equal(idx, ref[0]) and np.array_equal(sc, ref[1])
    for i in range(0, nq, 16):
        oi, os_, _ = m.two_stage(Q[i], 1, 512, k)
        assert np.array_equal(idx[i, :len(oi)], oi) and np.array_equal(sc[i, :len(oi)], os_), i
    with pytest.raises(E.AesError) as ei:  # above the 32 warps a CTA can hold
        eng.retune(batch_warps=40)
    assert ei.value.code == E.AES_ERR_INVALID


def test_batched_equals_plain_and_long_rows():
    rows, cols = 6000, 700
    ptr, col, val = E.gen_matrix(E.GEN_GAMMA_DEG, rows, cols, 120, 700, seed=77)
    Q = queries(cols, 40, 3, signed=True)
    out = []
    for bt in (1, 128):
        eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=6, split=4, ck=256, k_max=50,
                     max_batch=40, batch_tile=bt)
        eng.Q_reset(Q)
        eng(k=50)
        out.append(eng.read_topk())
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_batched_tiny_and_zero_queries():
    rows, cols = 70, 96
    m, eng = make(rows, cols, E.GEN_UNIFORM_DEG, 1, 12, 5, 8, 0, 32, 64, 10, nq=20,
                  batch_tile=128)
    Q = queries(cols, 20, 8, signed=True)
    Q[3] = 0.0
    check_run(m, eng, Q, 32, 64, 10)


@pytest.mark.parametrize("case", ["uniform", "even_rows_low", "large_k", "absnormal"])
def test_fp32_only_exact_path(case):
    """aes_run_exact: FP32 score of every row + Top-K equals the FP32 oracle (sw_test path).
    The select reads only the rows above a bound taken from every S-th row's key; in
    "even_rows_low" every sampled row scores low, the bound admits too many rows, and the call
    falls back to the select over every row (counted as repaired); "large_k" has no room for a
    sample bound and selects over every row directly."""
    rows, cols, k = 30000, 1024, 100
    kind, p0, p1 = E.GEN_UNIFORM_DEG, 10, 30
    if case == "large_k":
        k = 1000
    if case == "absnormal":
        rows, cols, kind, p0, p1 = 40000, 500, E.GEN_FIXED_ABSNORMAL, 69, 0
    ptr, col, val = E.gen_matrix(kind, rows, cols, p0, p1, seed=51)
    if case == "even_rows_low":
        val = val.copy()
        even = np.repeat(np.arange(rows) % 2 == 0, np.diff(ptr).astype(np.int64))
        val[even] *= np.float32(1e-3)
    m = orc.Matrix(rows, cols, ptr, col, val, 8, 0)
    eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=8, quant=0, split=1, ck=256,
                 k_max=k, max_batch=2)
    Q = queries(cols, 2, 52, signed=(case != "even_rows_low"))
    eng.Q_reset(Q)
    eng.stats(reset=True)
    idx, sc, ns = eng.run_exact(k=k)
    allrows = np.arange(rows, dtype=np.uint32)
    for i in range(2):
        s = orc.rescore_f32(m.ptr, m.col, m.val, Q[i], allrows)
        ri, rs = orc.sort_tuples_f32(allrows, s)
        assert np.array_equal(idx[i], ri[:k]) and np.array_equal(sc[i], rs[:k])
    if case == "even_rows_low":
        assert eng.stats(reset=True)["repaired"] >= 1


@pytest.mark.parametrize("bits,quant,split,ck,k,nq", [(8, 0, 1, 4096, 1024, 3), (8, 1, 32, 2048, 1000, 20),
                                                      (4, 2, 8, 1024, 777, 17),
                                                      (6, 0, 64, 2048, 100, 20)])
def test_large_k_and_ck(bits, quant, split, ck, k, nq):
    # the final pass selects the K best of up to 4096 rescored candidates, then sorts only those
    rows, cols = 30000, 1024
    m, eng = make(rows, cols, E.GEN_UNIFORM_DEG, 10, 30, 31, bits, quant, split, ck, k, nq=nq)
    Q = queries(cols, nq, 4, signed=(quant == 0))
    eng.Q_reset(Q)
    eng(k=k)
    idx, sc = eng.read_topk()
    for i in range(nq):
        oi, os_, _ = m.two_stage(Q[i], split, ck, k)
        assert np.array_equal(idx[i, :len(oi)], oi), f"query {i}"
        assert np.array_equal(sc[i, :len(oi)], os_), f"query {i}"
    # FP32-only path with the same K
    ei, es, _ = eng.run_exact(k=k)
    for i in range(nq):
        s = orc.rescore_f32(m.ptr, m.col, m.val, Q[i], np.arange(rows, dtype=np.uint32))
        s = np.where(s == 0, np.float32(0), s)
        top = np.lexsort((-np.arange(rows, dtype=np.int64), -s.astype(np.float64)))[:k]
        assert np.array_equal(ei[i], top.astype(np.uint32)), f"exact query {i}"


@pytest.mark.parametrize("bits,quant,qq", [(8, 0, 0), (6, 0, 0), (4, 0, 0), (8, 1, 0), (4, 2, 0),
                                           (6, 0, 1)])
def test_query_quantiser_on_rounding_ties(bits, quant, qq):
    # query values placed on M * x / m = k + 1/2 (and one ulp either side): the device's integer
    # quantiser must round them as numpy's float64 arithmetic does
    rows, cols = 4000, 1024
    m, eng = make(rows, cols, E.GEN_UNIFORM_DEG, 10, 30, 77, bits, quant, 1, 256, 16,
                  query_quant=qq)
    M = ((1 << bits) - 1) // 2 if quant == 0 else (1 << bits) - 1
    rng = np.random.default_rng(bits * 10 + quant)
    for trial in range(3):
        mx = np.float32(rng.uniform(0.5, 3.0))
        k = rng.integers(0, M, cols)
        q = (mx * (k + 0.5) / M).astype(np.float32)
        nudge = rng.integers(-1, 2, cols).astype(np.int32)
        q = (q.view(np.int32) + nudge).view(np.float32)
        q = np.minimum(q, mx)
        q[0] = mx
        if quant == 0:
            q = q * np.where(rng.random(cols) < 0.5, -1, 1).astype(np.float32)
        got = eng.score_all(q)
        assert np.array_equal(got, m.keys(q, qq=qq)), f"trial {trial}"


@pytest.mark.parametrize("kind,rows,p0,p1,bits,quant,split", [
    (E.GEN_UNIFORM_DEG, 400000, 10, 30, 8, 0, 1),
    (E.GEN_UNIFORM_DEG, 400000, 10, 30, 6, 0, 32),
    (E.GEN_UNIFORM_DEG, 400000, 10, 30, 4, 2, 1),
    (E.GEN_GAMMA_DEG, 150000, 120, 700, 8, 1, 8),
])
def test_rows_across_range_boundaries_at_scale(kind, rows, p0, p1, bits, quant, split):
    """Matrices large enough that every warp's range spans several tiles, so thousands of rows
    cross a boundary between two warps' ranges (and long rows cross several tiles).  Every
    row's key and the two-stage results must equal the oracle's."""
    cols, k, ck = 1024, 100, 1024
    m, eng = make(rows, cols, kind, p0, p1, 61, bits, quant, split, ck, k, nq=2)
    Q = queries(cols, 2, 13, signed=(quant == 0))
    for q in Q:
        assert np.array_equal(eng.score_all(q), m.keys(q))
    check_run(m, eng, Q, split, ck, k)
