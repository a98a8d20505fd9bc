"""aes_retune: a resident matrix re-planned for another CK / split / sample stride / batch tile
gives the same results as a handle created with those parameters, and the oracle's."""
import numpy as np
import pytest

import oracle as orc
from acceles_gb300 import engine as E

pytestmark = pytest.mark.gpu


def _setup(rows=30000, cols=1024, bits=4, quant=1, seed=5):
    ptr, col, val = E.gen_matrix(E.GEN_GAMMA_DEG, rows, cols, 32, 512, seed=seed)
    return ptr, col, val, orc.Matrix(rows, cols, ptr, col, val, bits, quant)


def _queries(cols, nq, seed):
    rng = np.random.default_rng(seed)
    Q = rng.random((nq, cols)).astype(np.float32)
    dens = rng.uniform(0.05, 0.30, nq)
    Q[rng.random((nq, cols)) >= dens[:, None]] = 0.0
    return Q


@pytest.mark.parametrize("ck,split,stride,tile,nq", [(256, 1, 4, 1, 3), (512, 32, 16, 128, 20),
                                                      (1024, 8, 0, 0, 20), (128, 1, 1, 128, 17)])
def test_retune_matches_fresh_handle_and_oracle(ck, split, stride, tile, nq):
    rows, cols, k = 30000, 1024, 100
    ptr, col, val, m = _setup(rows, cols)
    Q = _queries(cols, nq, 3)
    eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=4, quant=1, split=1, ck=1024,
                 k_max=k, max_batch=4)
    eng.Q_reset(Q[:4])
    eng(k=k)
    eng.retune(ck=ck, split=split, sample_stride=stride, batch_tile=tile, max_batch=nq)
    inf = eng.info()
    assert inf["split"] == split and inf["max_batch"] == nq
    eng.Q_reset(Q)
    eng(k=k)
    idx, sc = eng.read_topk()
    fresh = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=4, quant=1, split=split, ck=ck,
                   k_max=k, max_batch=nq, sample_stride=stride, batch_tile=tile)
    fresh.Q_reset(Q)
    fresh(k=k)
    fi, fs = fresh.read_topk()
    assert np.array_equal(idx, fi) and np.array_equal(sc, fs)
    for i in range(nq):
        oi, os_, _ = m.two_stage(Q[i], split, ck, k)
        assert np.array_equal(idx[i, :len(oi)], oi)
        assert np.array_equal(sc[i, :len(oi)], os_)


def test_retune_rejects_packing_changes_and_keeps_working():
    rows, cols, k = 20000, 1024, 50
    ptr, col, val, m = _setup(rows, cols, bits=4, quant=1)
    eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=4, quant=1, split=1, ck=512,
                 k_max=k)
    Q = _queries(cols, 1, 8)
    for bad in ({"bits": 8}, {"quant": 0}, {"pack_parts": 4}):
        with pytest.raises(E.AesError) as ei:
            eng.retune(**bad)
        assert ei.value.code == E.AES_ERR_INVALID
    # over the memory limit: refused before freeing, the old configuration still serves
    with pytest.raises(E.AesError) as ei:
        eng.retune(mem_limit=1 << 20)
    assert ei.value.code == E.AES_ERR_NOMEM
    eng.Q_reset(Q)
    eng(k=k)
    idx, sc = eng.read_topk()
    oi, os_, _ = m.two_stage(Q[0], 1, 512, k)
    assert np.array_equal(idx[0, :len(oi)], oi) and np.array_equal(sc[0, :len(oi)], os_)
    # a retune drops loaded queries
    eng.retune(ck=256)
    with pytest.raises(E.AesError) as ei:
        eng(k=k)
    assert ei.value.code == E.AES_ERR_STATE


def test_autotune_reaches_target_and_leaves_handle_tuned():
    from acceles_gb300 import autotune as AT
    rows, cols, k = 40000, 1024, 100
    ptr, col, val, m = _setup(rows, cols)
    eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=4, quant=1, split=1, ck=1024,
                 k_max=k, max_batch=32, flags=E.FLAG_TENSOR)
    Q = AT.sparse_queries(24, cols, 17)
    res = AT.tune(eng, Q, k, ck_ladder=(128, 256, 512, 1024, 2048), splits=(1, 32),
                  strides=(0, 16), reps=1)
    prm = res["params"]
    assert eng.info()["split"] == prm["split"]
    # every candidate pass of the grid was timed (plain, dp4a at 16, 12 and 8 warps per CTA,
    # tensor cores); the handle runs the chosen one
    assert {(t["batch_tile"], t["tensor"], t["batch_warps"]) for t in res["time_trials"]} == set(AT.PASSES)
    inf = eng.info()
    assert inf["tensor_tiles"] == (1 if prm["flags"] & E.FLAG_TENSOR else 0)
    if prm["batch_tile"] == 128 and not inf["tensor_tiles"]:
        assert inf["batch_warps"] > 0
        if prm["batch_warps"]:
            assert inf["batch_warps"] == prm["batch_warps"]
    # the chosen configuration reproduces the FP32-only Top-K on every sample query
    eng.Q_reset(Q)
    eng(k=k)
    idx, sc = eng.read_topk()
    assert np.array_equal(idx, res["exact"])
    # and matches the oracle's two-stage result for the chosen CK / split
    for i in range(3):
        oi, os_, _ = m.two_stage(Q[i], prm["split"], prm["ck"], k)
        assert np.array_equal(idx[i, :len(oi)], oi) and np.array_equal(sc[i, :len(oi)], os_)
    # the CK trial before the chosen one (same split) missed the target
    trials = [t for t in res["ck_trials"] if t["split"] == prm["split"]]
    assert trials[-1]["ck"] == prm["ck"] and trials[-1]["frac_identical"] == 1.0
    assert all(t["frac_identical"] < 1.0 for t in trials[:-1])


def test_retune_drops_captured_graphs():
    """A handle that replays CUDA graphs re-captures after a retune (the old graphs point at
    freed buffers) and gives the fresh handle's results."""
    rows, cols, k = 25000, 1024, 64
    ptr, col, val, m = _setup(rows, cols)
    Q = _queries(cols, 24, 12)
    eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=4, quant=1, split=1, ck=512,
                 k_max=k, max_batch=24, flags=E.FLAG_GRAPHS)
    for _ in range(2):  # capture, then replay
        eng.Q_reset(Q)
        eng(k=k)
    eng.retune(ck=256, split=8, sample_stride=16)
    for _ in range(2):
        eng.Q_reset(Q)
        eng(k=k)
    idx, sc = eng.read_topk()
    fresh = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=4, quant=1, split=8, ck=256,
                   k_max=k, max_batch=24, sample_stride=16)
    fresh.Q_reset(Q)
    fresh(k=k)
    fi, fs = fresh.read_topk()
    assert np.array_equal(idx, fi) and np.array_equal(sc, fs)


def test_autotune_ck_equals_oracle_brute_force():
    """The tuner's CK per split is the smallest of its ladder whose two-stage Top-K equals the
    FP32 exact Top-K on every sample query, both computed here by the oracle alone; the chosen
    pass is the fastest of the timed trials."""
    from acceles_gb300 import autotune as AT
    rows, cols, k, nq = 30000, 1024, 100, 20
    ptr, col, val, m = _setup(rows, cols, bits=8, quant=0, seed=9)
    eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=8, quant=0, split=1, ck=1024,
                 k_max=k, max_batch=nq)
    Q = _queries(cols, nq, 29)
    ladder, splits = (64, 128, 256, 512, 1024), (1, 32)
    res = AT.tune(eng, Q, k, ck_ladder=ladder, splits=splits, strides=(0, 16), reps=1,
                  passes=((1, False), (128, False), (128, False, 8)))
    xi, _ = orc.topk_f32_many(m.ptr, m.col, m.val, rows, cols, Q, k)
    for split in splits:
        want = None
        for ck in ladder:
            if ck < split:
                continue
            oi, _, on = orc.two_stage_many(m, Q, split, ck, k)
            if all(np.array_equal(oi[i, :on[i]], xi[i, :on[i]]) and on[i] == k for i in range(nq)):
                want = ck
                break
        got = [t["ck"] for t in res["ck_trials"] if t["split"] == split]
        assert want is not None and got[-1] == want, (split, got, want)
    best = min(res["time_trials"], key=lambda t: t["ms_per_query"])
    assert res["params"]["ck"] == best["ck"] and res["params"]["split"] == best["split"]
    assert res["params"]["batch_tile"] == best["batch_tile"]
    assert res["params"]["sample_stride"] == best["sample_stride"]
    assert res["params"]["batch_warps"] == best["batch_warps"]
