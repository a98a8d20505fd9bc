"""Serving loop: continuous batching over several resident matrices gives each request the same
result as running it alone; admission by memory refuses a matrix that does not fit; CUDA-graph
replay equals direct launches."""
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
    srv = Server()
    data = {}
    for name, kind, rows, cols, p0, p1, bits in _mats():
        ptr, col, val = E.gen_matrix(kind, rows, cols, p0, p1, seed=len(name) + rows)
        srv.add_matrix(name, rows, cols, ptr, col, val, max_batch=64, k_max=100, bits=bits,
                       split=1, ck=512)
        data[name] = (rows, cols, ptr, col, val, bits)
    srv.start()
    rng = np.random.default_rng(3)
    reqs = []
    for i in range(240):
        name = "abc"[int(rng.integers(3))]
        q = rng.random(data[name][1]).astype(np.float32)
        k = int([8, 32, 100][int(rng.integers(3))])
        reqs.append((name, q, k))
    futs = [None] * len(reqs)

    def client(lo, hi):
        for i in range(lo, hi):
            futs[i] = srv.submit(*reqs[i])

    th = [threading.Thread(target=client, args=(j * 60, (j + 1) * 60)) for j in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    mixed = [f.result(timeout=120) for f in futs]
    batched = sum(m.batches for m in srv.mats.values())
    srv.close()
    assert batched < len(reqs)  # requests really were batched together
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
    srv = Server(mem_budget=64 << 20)
    srv.add_matrix("small", 100000, 1024, ptr, col, val, max_batch=8, bits=8, split=1, ck=256)
    big = E.gen_matrix(E.GEN_UNIFORM_DEG, 2_000_000, 1024, 10, 30, seed=2)
    with pytest.raises(E.AesError) as ei:
        srv.add_matrix("big", 2_000_000, 1024, *big, max_batch=8, bits=8, split=1, ck=256)
    assert ei.value.code == E.AES_ERR_NOMEM
    srv.close()


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
