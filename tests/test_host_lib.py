"""CPU tests of the C-ABI library: it loads, exports every declared entry point, and its host
logic (generator, quantiser + Ultra-CSR packer) matches the oracle byte for byte.  No GPU."""
import os
import re

import numpy as np
import pytest

import oracle as orc
from acceles_gb300 import engine as E

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(REPO, "include", "acceles.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(aes_[a-z_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = E.load()
    decl = declared_symbols()
    assert set(decl) == set(E.EXPORTS)
    for name in decl:
        assert hasattr(L, name), name


def test_generator_deterministic_and_sorted():
    a = E.gen_matrix(E.GEN_UNIFORM_DEG, 2000, 1024, 10, 30, seed=7)
    b = E.gen_matrix(E.GEN_UNIFORM_DEG, 2000, 1024, 10, 30, seed=7)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    ptr, col, val = a
    deg = np.diff(ptr.astype(np.int64))
    assert deg.min() >= 10 and deg.max() <= 30
    for r in range(0, 2000, 97):
        c = col[ptr[r]:ptr[r + 1]]
        assert np.all(np.diff(c.astype(np.int64)) > 0)  # distinct, sorted
    assert val.min() >= 0.0 and val.max() < 1.0
    g = E.gen_matrix(E.GEN_GAMMA_DEG, 5000, 1024, 32, 512, seed=3)
    d = np.diff(g[0].astype(np.int64))
    assert d.min() >= 1 and d.max() <= 512 and 25 < d.mean() < 40
    n = E.gen_matrix(E.GEN_FIXED_ABSNORMAL, 300, 500, 69, 0, seed=1)
    assert np.all(np.diff(n[0].astype(np.int64)) == 69) and n[2].min() >= 0


def _packer_case(rows, cols, kind, p0, p1, bits, quant, seed, parts=32):
    ptr, col, val = E.gen_matrix(kind, rows, cols, p0, p1, seed=seed)
    pk, trb = E.pack_host(ptr, col, val, rows, cols, bits=bits, quant=quant, pack_parts=parts)
    m = orc.Matrix(rows, cols, ptr, col, val, bits, quant, parts=parts)
    ref = m.packets()
    assert pk.shape == ref.shape
    assert np.array_equal(pk, ref)
    # tile row bases are prefix counts of the flag bits
    P = orc.packet_size(bits)
    flags = np.array([orc.unpack_packet(p, bits, quant == 0)[0] for p in ref], dtype=object)
    nf = np.array([bin(int(f)).count("1") for f in flags], np.int64)
    tiles = (len(ref) + 31) // 32
    pref = np.concatenate([[0], np.cumsum([nf[t * 32:(t + 1) * 32].sum() for t in range(tiles)])])
    assert np.array_equal(trb.astype(np.int64), pref)
    assert pref[-1] == rows - 1
    return m, ref


@pytest.mark.parametrize("bits", [4, 6, 8])
@pytest.mark.parametrize("quant", [0, 1, 2])
def test_packer_matches_oracle(bits, quant):
    _packer_case(1000, 1024, E.GEN_UNIFORM_DEG, 10, 30, bits, quant, seed=bits * 10 + quant)


def test_packer_ragged_partitions_and_long_rows():
    # rows not divisible by 32, rows spanning many packets and tiles, tiny partitions
    _packer_case(77, 1024, E.GEN_GAMMA_DEG, 200, 1024, 6, 0, seed=5)
    _packer_case(5, 64, E.GEN_FIXED_UNIFORM, 64, 0, 8, 0, seed=6)
    _packer_case(1, 1024, E.GEN_FIXED_UNIFORM, 1024, 0, 4, 2, seed=9, parts=1)


def test_packer_decodes_back_to_quantised_csr():
    rows, cols, bits = 300, 700, 6
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, rows, cols, 1, 40, seed=11)
    m = orc.Matrix(rows, cols, ptr, col, val, bits, 0)
    ref = m.packets()
    P = orc.packet_size(bits)
    rowc, colc, valc = [], [], []
    base = 0
    first = True
    for p in ref:
        f, c, v = orc.unpack_packet(p, bits, True)
        ctr = orc.xdecode(f, P, base)
        base = int(ctr[-1])
        for j in range(P):
            if v[j] == 0 and c[j] == 0 and not (f >> j) & 1:
                continue  # tail slot
            rowc.append(int(ctr[j]))
            colc.append(int(c[j]))
            valc.append(int(v[j]))
    qrow = np.repeat(np.arange(rows), np.diff(m.qptr.astype(np.int64)))
    assert np.array_equal(np.array(rowc), qrow)
    assert np.array_equal(np.array(colc), m.qcol)
    assert np.array_equal(np.array(valc), m.qval)


def test_packet_known_answer():
    """Two rows, hand-computed bit positions for B=6 (P=30): flags at bits [0,30), columns at
    [30+10j, ...), values at [330+6j, ...)."""
    ptr = np.array([0, 2, 3], np.uint64)
    col = np.array([5, 1023, 7], np.uint32)
    val = np.array([1.0, -0.5, 0.25], np.float32)
    pk, _ = E.pack_host(ptr, col, val, 2, 1024, bits=6, quant=0, pack_parts=1)
    assert pk.shape == (1, 64)
    bits = np.unpackbits(pk[0], bitorder="little")
    # scale m = 1.0, M = 31: values 31, round(-15.5) = -16 (half to even), round(7.75) = 8
    assert list(bits[:3]) == [0, 0, 1]                     # row flags
    def field(pos, w):
        return int(sum(int(bits[pos + i]) << i for i in range(w)))
    assert field(30, 10) == 5 and field(40, 10) == 1023 and field(50, 10) == 7
    assert field(330, 6) == 31 and field(336, 6) == (-16) & 63 and field(342, 6) == 8
    assert bits[348:].sum() == 0 and bits[3:30].sum() == 0


def test_invalid_arguments_return_codes():
    ptr = np.array([0, 1], np.uint64)
    col = np.array([0], np.uint32)
    val = np.array([1.0], np.float32)
    with pytest.raises(E.AesError) as ei:
        E.pack_host(ptr, col, val, 1, 2048, bits=6)
    assert ei.value.code == E.AES_ERR_UNSUPPORTED
    with pytest.raises(E.AesError) as ei:
        E.pack_host(ptr, col, val, 1, 4, bits=5)
    assert ei.value.code == E.AES_ERR_UNSUPPORTED
    with pytest.raises(E.AesError) as ei:
        E.pack_host(ptr, col, -val, 1, 4, bits=6, quant=1)
    assert ei.value.code == E.AES_ERR_INVALID
    with pytest.raises(E.AesError):
        E.pack_host(ptr, np.array([9], np.uint32), val, 1, 4, bits=6)


def test_create_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(E.AesError) as ei:
        E.SpMV(2, 4, row=[0, 1], col=[0, 1], val=[1.0, 1.0])
    assert ei.value.code in (E.AES_ERR_NODEV, E.AES_ERR_CUDA)


def test_baseline_library_exports_its_header():
    from acceles_gb300 import gpu_baseline as G
    src = open(os.path.join(REPO, "include", "acceles_baseline.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    decl = set(re.findall(r"\b(aes_[a-z_]+)\s*\(", src))
    assert decl == set(G.EXPORTS)
    L = G.load()
    for name in decl:
        assert hasattr(L, name), name


def _e4m3_value(b):
    """Value of an FP8 e4m3 byte from the format: sign, 4-bit exponent biased by 7, 3-bit
    mantissa (normal numbers; subnormals 2^-6 * m/8)."""
    s = -1.0 if b & 0x80 else 1.0
    e, m = (b >> 3) & 15, b & 7
    return s * (2.0 ** (e - 7) * (1 + m / 8) if e else 2.0 ** -6 * m / 8)


@pytest.mark.parametrize("quant,cols,rows", [(orc.QUANT_SYM_GLOBAL, 1024, 700),
                                             (orc.QUANT_UNSIGNED_ROW, 500, 300),
                                             (orc.QUANT_UNSIGNED_GLOBAL, 200, 257)])
def test_tensor_tile_layout_decodes_to_quantised_matrix(quant, cols, rows):
    """Every entry of the tensor-core layout names its (row, column) through the operand offset
    and holds the quantised value exactly in e4m3; together they are the oracle's quantised
    matrix, each entry once, in the (tile, chunk) slot its row and column fall in."""
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, rows, cols, 3, 40, seed=cols)
    if quant == orc.QUANT_SYM_GLOBAL:
        val = (val * 2 - 1).astype(np.float32)
    m = orc.Matrix(rows, cols, ptr, col, val, 4, quant)
    tp, ent = E.pack_tc_host(ptr, col, val, rows, cols, bits=4, quant=quant, flags=E.FLAG_TENSOR)
    nch = ((cols + 31) // 32 * 32 + 255) // 256
    ntile = (rows + 127) // 128
    assert len(tp) == ntile * nch + 1 and tp[0] == 0 and len(ent) == len(m.qcol) == tp[-1]
    got = set()
    for t in range(ntile):
        for c in range(nch):
            for e in ent[tp[t * nch + c]:tp[t * nch + c + 1]]:
                off, b = int(e) >> 16, int(e) & 0xFF
                assert int(e) & 0xFF00 == 0
                kk, rem = divmod(off, 2048)
                rg, rem = divmod(rem, 128)
                rl, kl = divmod(rem, 16)
                r, k = rg * 8 + rl, kk * 16 + kl
                assert r < 128 and k < 256
                got.add((t * 128 + r, c * 256 + k, _e4m3_value(b)))
    # each chunk begins with one entry per bank present: one warp store hits distinct banks
    for j in range(len(tp) - 1):
        banks = (ent[tp[j]:tp[j + 1]] >> 18) & 31
        head = banks[:32]
        assert len(set(head.tolist())) == min(32, len(set(banks.tolist())))
    qv = m.qval.astype(np.int64)
    want = set()
    for r in range(rows):
        for i in range(int(m.qptr[r]), int(m.qptr[r + 1])):
            want.add((r, int(m.qcol[i]), float(qv[i])))
    assert got == want and len(want) == len(ent)


def test_tensor_tile_layout_only_for_4bit_without_repeats():
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, 300, 64, 3, 6, seed=2)
    for bits in (6, 8):
        tp, ent = E.pack_tc_host(ptr, col, val, 300, 64, bits=bits, quant=1, flags=E.FLAG_TENSOR)
        assert len(ent) == 0
    tp, ent = E.pack_tc_host(ptr, col, val, 300, 64, bits=4, quant=1, flags=0)
    assert len(ent) == 0
    # row 5 holds its first column twice (sorted CSR with a repeat)
    p = ptr.astype(np.int64)
    col2 = np.insert(col, p[5] + 1, col[p[5]])
    val2 = np.insert(val, p[5] + 1, np.float32(0.5))
    ptr2 = ptr.copy()
    ptr2[6:] += 1
    tp, ent = E.pack_tc_host(ptr2, col2, val2, 300, 64, bits=4, quant=1, flags=E.FLAG_TENSOR)
    assert len(ent) == 0


@pytest.mark.parametrize("kind,rows,cols,p0,p1", [
    (E.GEN_UNIFORM_DEG, 5000, 1024, 10, 30), (E.GEN_FIXED_ABSNORMAL, 3000, 500, 69, 0),
    (E.GEN_GAMMA_DEG, 4000, 1024, 32, 512), (E.GEN_FIXED_UNIFORM, 2000, 900, 108, 0),
    (E.GEN_UNIFORM_DEG, 500, 64, 40, 60)])
def test_oracle_generator_equals_engine_generator(kind, rows, cols, p0, p1):
    # the CPU baseline builds its inputs with the oracle's copy of the generator; both must give
    # the same matrix for the same arguments, whatever the thread count
    a = E.gen_matrix(kind, rows, cols, p0, p1, seed=11)
    for nt in (1, 3):
        b = orc.gen_matrix(kind, rows, cols, p0, p1, seed=11, nthreads=nt)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
