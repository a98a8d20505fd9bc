"""The no-allocation entry point (aes_run_noalloc) against the regular device entry point.

Some callers cannot allocate device memory once they serve queries (a latency-critical loop
that must not block or synchronise in cudaMalloc, or a process whose free memory is held by
another allocator).  aes_run_noalloc keeps its per-query scratch in a fixed device array inside
the library; this test checks, through the C ABI, that two calls in a row give the same Top-K
as aes_run_device, and that a matrix whose scratch would not fit is refused.
"""
import numpy as np
import pytest

from acceles_gb300 import engine as E

pytestmark = pytest.mark.gpu

RTOL = 1e-5  # exact-pass tolerance used by the parity tests


def test_noalloc_matches_run_device_twice():
    import torch
    rows, cols, k = 200_000, 1024, 100
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, rows, cols, 10, 30, seed=99)
    eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=8, split=1, ck=1024, k_max=k,
                 max_batch=2, batch_tile=1)
    Q = np.random.default_rng(5).random((2, cols)).astype(np.float32)
    dq = torch.from_numpy(Q).cuda()
    ref_i = torch.empty((2, k), dtype=torch.int32, device="cuda")
    ref_s = torch.empty((2, k), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    eng.run_device(dq.data_ptr(), 2, k, ref_i.data_ptr(), ref_s.data_ptr(), stream.cuda_stream)
    eng.finish()
    torch.cuda.synchronize()
    for q in range(2):  # two calls in a row share the scratch array
        oi = torch.full((k,), -1, dtype=torch.int32, device="cuda")
        os_ = torch.zeros((k,), dtype=torch.float32, device="cuda")
        eng.run_noalloc(dq[q].data_ptr(), k, oi.data_ptr(), os_.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize()
        gi, gs = oi.cpu().numpy(), os_.cpu().numpy()
        ri, rs = ref_i[q].cpu().numpy(), ref_s[q].cpu().numpy()
        assert np.array_equal(gi, ri)
        assert np.allclose(gs, rs, rtol=RTOL, atol=0)


def test_noalloc_rejects_scratch_over_limit():
    import torch
    # every tile sampled: 5M sample keys (20 MB) exceed the 16 MiB scratch
    rows, cols = 5_000_000, 64
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, rows, cols, 1, 3, seed=3)
    eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=8, split=1, ck=64, k_max=10,
                 sample_stride=1)
    dq = torch.rand(cols, device="cuda")
    oi = torch.empty(10, dtype=torch.int32, device="cuda")
    os_ = torch.empty(10, dtype=torch.float32, device="cuda")
    with pytest.raises(E.AesError) as ei:
        eng.run_noalloc(dq.data_ptr(), 10, oi.data_ptr(), os_.data_ptr())
    assert ei.value.code == E.AES_ERR_UNSUPPORTED


def test_noalloc_exact_slow_path_matches_oracle():
    # Scores decreasing with the row index put the global top rows in the first (sampled) tile,
    # so the sample threshold admits too few rows and the entry point repairs the query on its
    # exact slow path (every row's key, the select over all of them, the FP32 rescoring); two
    # calls in a row, each checked against the oracle
    import torch
    import oracle as orc
    rows, cols, k, ck = 40000, 256, 100, 512
    ptr = np.arange(rows + 1, dtype=np.uint64) * 4
    col = np.tile(np.array([0, 1, 2, 3], np.uint32), rows)
    val = np.repeat(np.linspace(1.0, 0.01, rows).astype(np.float32), 4)
    m = orc.Matrix(rows, cols, ptr, col, val, 8, orc.QUANT_SYM_GLOBAL)
    eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=8, split=1, ck=ck, k_max=k,
                 sample_stride=4)
    q = np.ones(cols, np.float32)
    oi_ref, os_ref, _ = m.two_stage(q, 1, ck, k)
    dq = torch.from_numpy(q).cuda()
    eng.stats(reset=True)
    for _ in range(2):
        oi = torch.full((k,), -1, dtype=torch.int32, device="cuda")
        os_ = torch.zeros((k,), dtype=torch.float32, device="cuda")
        eng.run_noalloc(dq.data_ptr(), k, oi.data_ptr(), os_.data_ptr())
        torch.cuda.synchronize()
        gi = oi.cpu().numpy().view(np.uint32)
        gs = os_.cpu().numpy()
        assert np.array_equal(gi[:len(oi_ref)], oi_ref)
        assert np.allclose(gs[:len(os_ref)], os_ref, rtol=RTOL, atol=0)
    st = eng.stats(reset=True)
    assert st["repaired"] == 2 and st["cand_launches"] == 4 and st["launches"] >= 12


def test_noalloc_rejects_negative_query_under_unsigned_quantiser():
    import torch
    rows, cols = 1000, 64
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, rows, cols, 2, 6, seed=1)
    eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, bits=8, quant=E.QUANT_UNSIGNED_ROW,
                 split=1, ck=64, k_max=10)
    dq = -torch.ones(cols, device="cuda")
    oi = torch.empty(10, dtype=torch.int32, device="cuda")
    os_ = torch.empty(10, dtype=torch.float32, device="cuda")
    with pytest.raises(E.AesError) as ei:
        eng.run_noalloc(dq.data_ptr(), 10, oi.data_ptr(), os_.data_ptr())
    assert ei.value.code == E.AES_ERR_QUERY
