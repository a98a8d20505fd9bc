"""Serving loop: continuous batching over several resident matrices, with two batches of one
matrix on the GPU at once, gives each request the same result as running it alone; admission by
memory refuses a matrix, or a batch slot, that does not fit; a view shares its base's matrix;
CUDA-graph replay equals direct launches."""
import threading

import numpy as np
import pytest

from acceles_gb300 import engine as E
from acceles_gb300.serve import Server

pytestmark = pytest.mark.gpu


def _mats():
    return [("a", E.GEN_UNIFORM_DEG, 40000, 1024, 10, 30, 8),
            ("b", E.GEN_FIXED_UNIFORM, 8000, 900, 108, 0, 8),
            ("c", E.GEN_GAMMA_DEG, 30000, 512, 32, 512, 6)]


def test_results_same_alone_and_in_the_mix():
    # two batch slots per matrix (the handle and a view); every request is queued before the
    # workers start, so both slots of a matrix take batches at once and overlap on the GPU
    srv = Server(slots=2)
    data = {}
    for name, kind, rows, cols, p0, p1, bits in _mats():
        ptr, col, val = E.gen_matrix(kind, rows, cols, p0, p1, seed=len(name) + rows)
        info = srv.add_matrix(name, rows, cols, ptr, col, val, max_batch=16, k_max=100,
                              bits=bits, split=1, ck=512)
        assert info["slots"] == 2
        data[name] = (rows, cols, ptr, col, val, bits)
    rng = np.random.default_rng(3)
    reqs = []
    for i in range(240):
        name = "abc"[int(rng.integers(3))]
        q = rng.random(data[name][1]).astype(np.float32)
        k = int([8, 32, 100][int(rng.integers(3))])
        reqs.append((name, q, k))
    futs = [srv.submit(*r) for r in reqs]
    srv.start()
    # more requests from client threads while batches are on the GPU
    extra = []
    for i in range(60):
        name = "abc"[int(rng.integers(3))]
        extra.append((name, rng.random(data[name][1]).astype(np.float32), 100))
    efuts = [None] * len(extra)

    def client(lo, hi):
        for i in range(lo, hi):
            efuts[i] = srv.submit(*extra[i])

    th = [threading.Thread(target=client, args=(j * 15, (j + 1) * 15)) for j in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    reqs += extra
    mixed = [f.result(timeout=120) for f in futs + efuts]
    batched = sum(m.batches for m in srv.mats.values())
    overlap = max(m.max_in_flight for m in srv.mats.values())
    srv.close()
    assert batched < len(reqs)  # requests really were batched together
    assert overlap >= 2  # two batches of one matrix ran at the same time
    alone = {}
    for name, (rows, cols, ptr, col, val, bits) in data.items():
        alone[name] = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=bits, split=1, ck=512,
                             k_max=100, max_batch=1)
    for (name, q, k), (gi, gs, _) in zip(reqs, mixed):
        e = alone[name]
        e.Q_reset(q)
        e(k=k)
        ai, asc = e.read_topk()
        assert np.array_equal(gi, ai[0]) and np.array_equal(gs, asc[0])


def test_admission_by_memory():
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, 100000, 1024, 10, 30, seed=1)
    kw = dict(max_batch=64, bits=8, split=1, ck=256)
    probe = E.SpMV(100000, 1024, ptr=ptr, col=col, val=val, k_max=100, **kw)
    base_b = probe.info()["device_bytes"]
    view = probe.view()
    view_b = view.info()["device_bytes"]
    view.close()
    probe.close()
    assert 0 < view_b < base_b
    # room for the matrix and one batch slot, not for a second slot
    srv = Server(mem_budget=base_b + view_b // 2, slots=2)
    info = srv.add_matrix("small", 100000, 1024, ptr, col, val, **kw)
    assert info["slots"] == 1
    big = E.gen_matrix(E.GEN_UNIFORM_DEG, 2_000_000, 1024, 10, 30, seed=2)
    with pytest.raises(E.AesError) as ei:
        srv.add_matrix("big", 2_000_000, 1024, *big, **kw)
    assert ei.value.code == E.AES_ERR_NOMEM
    srv.close()


def test_view_shares_the_matrix_and_outlives_its_base():
    rows, cols = 60000, 1024
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, rows, cols, 10, 30, seed=21)
    Q = np.random.default_rng(5).random((20, cols)).astype(np.float32)
    base = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=8, split=1, ck=512, k_max=100,
                  max_batch=20)
    view = base.view(ck=1024)
    assert view.info()["device_bytes"] < base.info()["device_bytes"]
    base.Q_reset(Q)
    base(k=100)
    bi, bs = base.read_topk()
    base.close()  # the matrix stays resident for the view
    view.retune(ck=512)
    view.Q_reset(Q)
    view(k=100)
    vi, vs = view.read_topk()
    assert np.array_equal(bi, vi) and np.array_equal(bs, vs)
    view.close()


def test_graph_replay_equals_direct_launches():
    rows, cols = 50000, 1024
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, rows, cols, 10, 30, seed=8)
    Q = np.random.default_rng(4).random((40, cols)).astype(np.float32)
    outs = []
    for flags in (0, E.FLAG_GRAPHS):
        eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=8, split=1, ck=1024,
                     k_max=100, max_batch=40, flags=flags)
        for rep in range(2):  # second run replays the captured graph
            eng.Q_reset(Q)
            eng(k=100)
            outs.append(tuple(x.copy() for x in eng.read_topk()))
    for o in outs[1:]:
        assert np.array_equal(o[0], outs[0][0]) and np.array_equal(o[1], outs[0][1])
