"""Row-sharded Top-K: merge the per-shard results of the two-stage method exactly.

The reference splits the rows into independent contiguous partitions (32 FPGA compute units,
host_spmv_ucsr.cpp:204-214, 280-286) and merges the units' candidates on the host
(Q_read_result, :691-748).  Across GPUs the same holds: each rank owns a contiguous block of
rows, keeps its local Top-CK by candidate key, rescores those rows in FP32, and sends
(key, row, fp32 score) triples.  Because every global Top-CK row is in its own shard's
Top-CK, selecting the global Top-CK by (key desc, row desc) among the gathered triples and then
the Top-K by (fp32 desc, row desc) reproduces the single-device result exactly.  With split > 1
the shards hold whole partitions and the per-partition candidates simply concatenate.

The exchange is one all-gather of CK triples per query (12 bytes each).
"""
from __future__ import annotations

import numpy as np


def _order_desc(primary, rows):
    """Indices sorting by (primary desc, row desc)."""
    return np.lexsort((-rows.astype(np.int64), -primary.astype(np.int64)))


def key_of_f32(x):
    """Order-preserving uint32 key of FP32 values (-0 and +0 equal)."""
    x = np.asarray(x, np.float32).copy()
    x[x == 0] = 0.0
    u = x.view(np.uint32)
    return np.where(u & 0x80000000, ~u, u | 0x80000000).astype(np.uint32)


def merge_shards(keys, rows, scores, ck, k):
    """Exact merge of gathered per-shard candidates of one query.

    keys/rows/scores: concatenation over shards of each shard's Top-CK candidate keys (uint32),
    global row ids (uint32) and FP32 exact scores.  Returns (rows[k'], scores[k']) of the global
    Top-K with k' = min(k, number of candidates), in (score desc, row desc) order.
    """
    keys = np.asarray(keys, np.uint32)
    rows = np.asarray(rows, np.uint32)
    scores = np.asarray(scores, np.float32)
    top = _order_desc(keys, rows)[:ck]
    r, s = rows[top], scores[top]
    o = _order_desc(key_of_f32(s), r)[:k]
    return r[o], s[o]


def shard_rows(rows: int, world: int, rank: int):
    """Contiguous row block [r0, r1) of a rank."""
    r0 = rows * rank // world
    r1 = rows * (rank + 1) // world
    return r0, r1


def gather_merge(local_keys, local_rows, local_scores, ck, k, group=None):
    """All-gather one query's local candidates over torch.distributed and merge them."""
    import torch
    import torch.distributed as dist

    n = torch.tensor([len(local_rows)], dtype=torch.int64)
    world = dist.get_world_size(group)
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    cap = int(max(s.item() for s in sizes))
    pad = np.zeros((3, cap), np.int64)
    m = len(local_rows)
    pad[0, :m] = np.asarray(local_keys, np.int64)
    pad[1, :m] = np.asarray(local_rows, np.int64)
    pad[2, :m] = np.asarray(local_scores, np.float32).view(np.int32).astype(np.int64)
    t = torch.from_numpy(pad)
    parts = [torch.zeros_like(t) for _ in range(world)]
    dist.all_gather(parts, t, group=group)
    ks, rs, ss = [], [], []
    for p, sz in zip(parts, sizes):
        q = p.numpy()[:, : int(sz.item())]
        ks.append(q[0].astype(np.uint32))
        rs.append(q[1].astype(np.uint32))
        ss.append(q[2].astype(np.int32).view(np.float32))
    return merge_shards(np.concatenate(ks), np.concatenate(rs), np.concatenate(ss), ck, k)
