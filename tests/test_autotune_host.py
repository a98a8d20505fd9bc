"""CPU tests of the autotuner's host logic with a stand-in engine (no GPU): the CK ladder stops
at the first CK whose Top-K equals the FP32-only Top-K, every candidate pass the handle offers
is timed, the tensor-core pass is skipped where the handle has no tile layout, and the handle
is left retuned to the fastest trial."""
import time
import types

import numpy as np
import pytest

from acceles_gb300 import autotune as AT
from acceles_gb300 import engine as E


class FakeEngine:
    """Records retune calls; Top-K is exact from `good_ck` on; a run sleeps per pass."""

    def __init__(self, layout, cost, good_ck=256, nq=8, k=5):
        self.params = types.SimpleNamespace(flags=E.FLAG_GRAPHS, ck=1024, split=1, batch_tile=0,
                                            sample_stride=0, max_batch=nq, k_max=k,
                                            batch_warps=0)
        self.layout, self.cost, self.good_ck, self.k = layout, cost, good_ck, k
        self.exact = np.arange(nq * k, dtype=np.uint32).reshape(nq, k)
        self.calls = []

    def retune(self, **kw):
        self.calls.append(dict(kw))
        for key, v in kw.items():
            setattr(self.params, key, v)

    def info(self):
        t = bool(self.params.flags & E.FLAG_TENSOR) and self.layout and self.params.batch_tile != 1
        w = (self.params.batch_warps or 16) if self.params.batch_tile != 1 else 0
        return {"tensor_tiles": 1 if t else 0, "split": self.params.split, "batch_warps": w}

    def Q_reset(self, q):
        self.nq = len(q)

    def run_exact(self, k):
        return self.exact[: self.nq], None, 0

    def __call__(self, k):
        tensor = self.info()["tensor_tiles"] == 1
        key = "tensor" if tensor else ("dp4a" if self.params.batch_tile == 128 else "plain")
        time.sleep(self.cost[key])
        return 0

    def read_topk(self):
        idx = self.exact[: self.nq].copy()
        if self.params.ck < self.good_ck:
            idx[0, 0] = 0xFFFFFFFE  # one query misses a row below the good CK
        return idx, None

    def stats(self, reset=False):
        return {"repaired": 0}


@pytest.mark.parametrize("layout,fastest", [(True, "tensor"), (False, "dp4a")])
def test_tune_times_every_pass_and_keeps_the_fastest(layout, fastest):
    eng = FakeEngine(layout, {"plain": 0.008, "dp4a": 0.004, "tensor": 0.001})
    Q = np.zeros((16, 8), np.float32)
    res = AT.tune(eng, Q, 5, ck_ladder=(128, 256, 512), strides=(0, 64), reps=1)
    # the ladder stopped at the first CK with the exact Top-K
    assert [t["ck"] for t in res["ck_trials"]] == [128, 256]
    assert res["params"]["ck"] == 256
    passes = {(t["batch_tile"], t["tensor"], t["batch_warps"]) for t in res["time_trials"]}
    want = {(1, False, 0), (128, False, 0), (128, False, 12), (128, False, 8)}
    want |= {(128, True, 0)} if layout else set()
    assert passes == want
    p = res["params"]
    assert (p["flags"] & E.FLAG_TENSOR != 0) == (fastest == "tensor")
    assert p["batch_tile"] == (1 if fastest == "plain" else 128)
    assert p["flags"] & E.FLAG_GRAPHS  # flags other than the tensor bit are kept
    # the handle is left on the chosen parameters
    assert eng.params.ck == 256 and eng.params.batch_tile == p["batch_tile"]
    assert eng.params.flags == p["flags"]


def test_tune_skips_batched_passes_below_16_queries():
    eng = FakeEngine(True, {"plain": 0.001, "dp4a": 0.0001, "tensor": 0.0001}, nq=8)
    Q = np.zeros((8, 8), np.float32)
    res = AT.tune(eng, Q, 5, ck_ladder=(256,), strides=(0,), reps=1)
    assert {t["batch_tile"] for t in res["time_trials"]} == {1}
    assert res["params"]["batch_tile"] == 1


def test_sparse_queries_density_and_seed():
    Q = AT.sparse_queries(200, 1024, 7)
    d = (Q != 0).mean(axis=1)
    assert d.min() > 0.02 and d.max() < 0.35
    assert np.array_equal(Q, AT.sparse_queries(200, 1024, 7))
    assert Q.min() >= 0.0 and Q.max() < 1.0
