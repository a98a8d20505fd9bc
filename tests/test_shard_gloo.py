"""Row-sharded Top-K over two CPU ranks (gloo): each rank keeps its shard's Top-CK by candidate
key, rescores it in FP32, and the all-gather merge reproduces the single-device two-stage
result exactly (acceles_gb300/shard.py)."""
import os
import socket

import numpy as np
import pytest

ROWS, COLS, CK, K = 6000, 256, 256, 50


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_dir):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.dirname(here))
    sys.path.insert(0, os.path.join(os.path.dirname(here), "oracle"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    import oracle as orc
    from acceles_gb300 import engine as E, shard
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, ROWS, COLS, 5, 25, seed=4)
    m = orc.Matrix(ROWS, COLS, ptr, col, val, 8, orc.QUANT_SYM_GLOBAL)
    r0, r1 = shard.shard_rows(ROWS, world, rank)
    res = []
    for qi in range(3):
        q = np.random.default_rng(qi).random(COLS).astype(np.float32)
        keys = m.keys(q)[r0:r1]
        rows = np.arange(r0, r1, dtype=np.uint32)
        sel = np.lexsort((-rows.astype(np.int64), -keys.astype(np.int64)))[:CK]
        lk, lr = keys[sel], rows[sel]
        ls = orc.rescore_f32(m.ptr, m.col, m.val, q, lr)
        gi, gs = shard.gather_merge(lk, lr, ls, CK, K)
        res.append((gi, gs))
    if rank == 0:
        np.save(os.path.join(out_dir, "merged.npy"),
                np.array([np.concatenate([a.astype(np.float64), b.astype(np.float64)]) for a, b in res]))
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_merge_matches_single_device(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import oracle as orc
    from acceles_gb300 import engine as E
    mp.spawn(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    got = np.load(tmp_path / "merged.npy")
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, ROWS, COLS, 5, 25, seed=4)
    m = orc.Matrix(ROWS, COLS, ptr, col, val, 8, orc.QUANT_SYM_GLOBAL)
    for qi in range(3):
        q = np.random.default_rng(qi).random(COLS).astype(np.float32)
        oi, os_, _ = m.two_stage(q, 1, CK, K)
        assert np.array_equal(got[qi][:K].astype(np.uint32), oi)
        assert np.array_equal(got[qi][K:].astype(np.float32), os_)


def test_merge_shards_unit():
    from acceles_gb300 import shard
    keys = np.array([5, 9, 9, 1, 7], np.uint32)
    rows = np.array([10, 3, 8, 2, 4], np.uint32)
    scores = np.array([0.5, 0.9, 0.1, 0.95, 0.9], np.float32)
    r, s = shard.merge_shards(keys, rows, scores, ck=3, k=2)
    # Top-3 by key: (9,8), (9,3), (7,4); by score: 0.9 rows 4 and 3 tie -> row desc
    assert list(r) == [4, 3] and np.allclose(s, [0.9, 0.9])
