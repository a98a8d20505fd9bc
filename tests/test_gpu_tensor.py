"""GPU parity of the tensor-core candidate pass of 4-bit matrices (tcgen05, FP8 e4m3 operands
holding the 4-bit integers exactly, FP32 accumulation): Top-K rows, FP32 scores and the
candidate set bit-exact with the CPU oracle, and equal to the dp4a batched pass on the same
handle."""
import numpy as np
import pytest

import oracle as orc
from acceles_gb300 import engine as E

pytestmark = pytest.mark.gpu


def queries(cols, nq, seed, signed):
    q = np.random.default_rng(seed).random((nq, cols)).astype(np.float32)
    return q * 2 - 1 if signed else q


def run(eng, Q, k):
    eng.Q_reset(Q)
    eng(k=k)
    idx, sc = eng.read_topk()
    cands = [eng.read_candidates(i)[0] for i in range(Q.shape[0])]
    return idx, sc, cands


# rows not a multiple of 128 (a partial last tile); cols covering one partial chunk (200),
# a partial last chunk (500, 900) and four full chunks (1024); 130 queries = a full block and
# a block of two, run by a CTA pair (two blocks per launch); 300 = a pair and a single block;
# the three quantisers; one and 32 partitions; three chunk buffers, and two where the
# thresholds of 32 partitions leave no room for a third (1024 columns); an odd number of row
# tiles (the last pair's second CTA has none); a matrix of one row tile on a pair
@pytest.mark.parametrize("rows,cols,quant,split,ck,nq", [
    (20000, 1024, 0, 1, 1024, 130),
    (12000, 1024, 1, 32, 512, 40),
    (12000, 1024, 1, 32, 512, 256),
    (12800 + 77, 1024, 1, 1, 256, 300),
    (9000, 500, 0, 4, 512, 256),
    (100, 64, 1, 1, 64, 200),
    (20000, 1024, 1, 1, 256, 128),
    (9000, 500, 2, 32, 512, 64),
    (7777, 200, 0, 32, 512, 20),
    (5000, 900, 1, 8, 256, 3),
])
def test_tensor_pass_matches_oracle(rows, cols, quant, split, ck, nq):
    k = 100
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, rows, cols, 10, 30, seed=rows + cols)
    m = orc.Matrix(rows, cols, ptr, col, val, 4, quant)
    eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=4, quant=quant, split=split, ck=ck,
                 k_max=k, max_batch=nq, batch_tile=128, flags=E.FLAG_TENSOR)
    assert eng.info()["tensor_tiles"] == 1
    Q = queries(cols, nq, 5, signed=(quant == 0))
    idx, sc, cands = run(eng, Q, k)
    for i in range(0, nq, max(1, nq // 7)):
        oi, os_, cand = m.two_stage(Q[i], split, ck, k)
        n = len(oi)
        assert np.array_equal(idx[i, :n], oi), i
        assert np.array_equal(sc[i, :n], os_), i
        keys = m.keys(Q[i])
        exp = cand[np.lexsort((-cand.astype(np.int64), -keys[cand].astype(np.int64)))]
        assert np.array_equal(cands[i], exp), i
    # the dp4a pass on the same handle returns the same candidates and Top-K
    eng.retune(flags=0)
    assert eng.info()["tensor_tiles"] == 0
    idx2, sc2, cands2 = run(eng, Q, k)
    assert np.array_equal(idx, idx2) and np.array_equal(sc, sc2)
    for a, b in zip(cands, cands2):
        assert np.array_equal(a, b)


def test_tensor_pass_long_rows_and_zero_query():
    """Gamma-degree rows up to the full width (every chunk of a tile populated), a zero query
    (every score 0: all rows tie) and the plain path for a small batch on the same handle."""
    rows, cols, k, nq = 6000, 1024, 50, 40
    ptr, col, val = E.gen_matrix(E.GEN_GAMMA_DEG, rows, cols, 200, 1024, seed=9)
    m = orc.Matrix(rows, cols, ptr, col, val, 4, 1)
    eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=4, quant=1, split=4, ck=256,
                 k_max=k, max_batch=nq, flags=E.FLAG_TENSOR)
    assert eng.info()["tensor_tiles"] == 1
    Q = queries(cols, nq, 3, signed=False)
    Q[7] = 0.0
    idx, sc, _ = run(eng, Q, k)
    for i in (0, 7, 21, 39):
        oi, os_, _ = m.two_stage(Q[i], 4, 256, k)
        n = len(oi)
        assert np.array_equal(idx[i, :n], oi), i
        assert np.array_equal(sc[i, :n], os_), i
    # 3 queries take the plain pass (batched from 16 queries on): same results
    idx3, sc3, _ = run(eng, Q[:3], k)
    assert np.array_equal(idx3, idx[:3]) and np.array_equal(sc3, sc[:3])


def test_tensor_layout_not_built_for_duplicates_or_wide_bits():
    """A row holding a column twice would lose one value in the dense tile: the layout is not
    built and the dp4a pass runs.  6- and 8-bit matrices ignore the flag."""
    rows, cols = 300, 64
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, rows, cols, 3, 6, seed=2)
    r = np.repeat(np.arange(rows, dtype=np.uint32), np.diff(ptr).astype(np.int64))
    c = col.astype(np.uint32).copy()
    v = val.astype(np.float32).copy()
    r = np.concatenate([r, np.array([5], np.uint32)])
    c = np.concatenate([c, c[ptr[5]:ptr[5] + 1]])
    v = np.concatenate([v, np.array([0.5], np.float32)])
    eng = E.SpMV(rows, cols, row=r, col=c, val=v, bits=4, quant=1, split=1, ck=64, k_max=10,
                 max_batch=20, flags=E.FLAG_TENSOR)
    assert eng.info()["tensor_tiles"] == 0
    for bits in (6, 8):
        e2 = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=bits, quant=1, split=1, ck=64,
                    k_max=10, max_batch=20, flags=E.FLAG_TENSOR)
        assert e2.info()["tensor_tiles"] == 0


@pytest.mark.parametrize("nq", [64, 200])
def test_tensor_pass_gives_up_and_recovers(nq):
    """The failure path of the pass's bounded waits: with the MMA role idle (a test flag) every
    hand-over wait of the producers and the epilogue runs out after about a second, the pass
    frees its tensor memory and the run returns AES_ERR_CUDA; the next ordinary run on the same
    handle is oracle-exact, so the context and the tensor memory are usable again.  200 queries
    run on CTA pairs: both CTAs of a pair give up and meet before they free tensor memory."""
    rows, cols, k, ck = 40000, 1024, 100, 256  # 313 row tiles: every CTA has two or more
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, rows, cols, 10, 30, seed=77)
    m = orc.Matrix(rows, cols, ptr, col, val, 4, orc.QUANT_UNSIGNED_ROW)
    eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=4, quant=E.QUANT_UNSIGNED_ROW,
                 split=1, ck=ck, k_max=k, max_batch=nq, flags=E.FLAG_TENSOR)
    assert eng.info()["tensor_tiles"] == 1
    Q = queries(cols, nq, 78, signed=False)
    eng.retune(flags=E.FLAG_TENSOR | E.FLAG_TEST_IDLE_MMA)
    eng.Q_reset(Q)
    with pytest.raises(E.AesError) as ex:
        eng(k=k)
    assert ex.value.code == E.AES_ERR_CUDA
    eng.retune(flags=E.FLAG_TENSOR)
    idx, sc, _ = run(eng, Q, k)
    for i in (0, nq - 1):
        oi, os_, _ = m.two_stage(Q[i], 1, ck, k)
        assert np.array_equal(idx[i, :len(oi)], oi) and np.array_equal(sc[i, :len(oi)], os_)


def test_tensor_pass_graph_replay_on_pairs():
    """A CUDA graph captured with the pair launches (clusters of two CTAs) replays to the same
    results as direct launches, for a batch of two blocks and one of three (a pair and a single
    CTA)."""
    rows, cols, k = 30000, 1024, 100
    ptr, col, val = E.gen_matrix(E.GEN_GAMMA_DEG, rows, cols, 32, 512, seed=91)
    for nq in (256, 300):
        Q = queries(cols, nq, 92, signed=False)
        out = []
        for flags in (E.FLAG_TENSOR, E.FLAG_TENSOR | E.FLAG_GRAPHS):
            eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=4, quant=E.QUANT_UNSIGNED_ROW,
                         split=1, ck=256, k_max=k, max_batch=nq, batch_tile=128, flags=flags)
            assert eng.info()["tensor_tiles"] == 1
            for _ in range(2):  # with graphs: capture, then replay
                eng.Q_reset(Q)
                eng(k=k)
                out.append(tuple(x.copy() for x in eng.read_topk()))
            eng.close()
        for o in out[1:]:
            assert np.array_equal(o[0], out[0][0]) and np.array_equal(o[1], out[0][1])
