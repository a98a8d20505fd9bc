"""Data formats on either side of the path (no GPU): Matrix Market files against the
reference's own readMtx, ReSparse against the reference's resparse_spm (golden fixtures) and
the oracle, and the keep-ratio bisection against the oracle's restatement of the reference
loop."""
import os

import numpy as np
import pytest

import oracle as orc
from acceles_gb300 import engine as E
from acceles_gb300 import resparse as RS

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _bits(a):
    return np.asarray(a, np.float32).view(np.uint32)


# ---- Matrix Market ----------------------------------------------------------------------------

def _mtx_cases():
    g = np.load(os.path.join(GOLD, "mtx.npz"))
    n = len([k for k in g.files if k.endswith("_args")])
    return [(g, i) for i in range(n)]


@pytest.mark.parametrize("case", range(len(_mtx_cases())))
def test_read_mtx_matches_reference_readMtx(case):
    g, i = _mtx_cases()[case]
    directed, read_values, zero, srt = (int(x) for x in g[f"c{i}_args"])
    name = str(g[f"c{i}_name"])
    flags = (E.MTX_KEEP_DIRECTED if directed == 1 else 0) | (E.MTX_ZERO_INDEXED if zero else 0) \
        | (E.MTX_SORT if srt else 0)
    rows, cols, r, c, v = E.read_mtx(os.path.join(GOLD, "mtx", name), flags)
    assert (rows, cols) == tuple(int(x) for x in g[f"c{i}_shape"])
    assert np.array_equal(r, g[f"c{i}_row"]) and np.array_equal(c, g[f"c{i}_col"])
    assert np.array_equal(_bits(v), _bits(g[f"c{i}_val"]))


@pytest.mark.parametrize("flags", [0, E.MTX_ZERO_INDEXED])
def test_mtx_round_trip_is_bit_exact(tmp_path, flags):
    rng = np.random.default_rng(4)
    n = 5000
    r = rng.integers(0, 300, n).astype(np.uint32)
    c = rng.integers(0, 70, n).astype(np.uint32)
    v = (rng.standard_normal(n) * 10.0 ** rng.integers(-30, 30, n)).astype(np.float32)
    v[:5] = [0.0, -0.0, 1.0, np.float32(1e-45), np.float32(3.4028235e38)]
    p = str(tmp_path / "m.mtx")
    E.write_mtx(p, 300, 70, r, c, v, flags)
    rows, cols, r2, c2, v2 = E.read_mtx(p, flags)
    assert (rows, cols) == (300, 70)
    assert np.array_equal(r, r2) and np.array_equal(c, c2)
    assert np.array_equal(_bits(v), _bits(v2))
    # sorted read: (row, col) order, equal keys in file order
    _, _, r3, c3, v3 = E.read_mtx(p, flags | E.MTX_SORT)
    o = np.lexsort((c.astype(np.int64), r.astype(np.int64)))
    assert np.array_equal(r3, r[o]) and np.array_equal(c3, c[o])
    assert np.array_equal(_bits(v3), _bits(v[o]))


@pytest.mark.parametrize("text", [
    "%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n",     # dense storage
    "%%MatrixMarket matrix coordinate complex general\n1 1 1\n1 1 1 0\n",
    "%MatrixMarket matrix coordinate real general\n1 1 1\n1 1 1\n",   # bad banner
    "%%MatrixMarket matrix coordinate real general\n3 3 2\n1 1 1\n",  # too few entries
    "%%MatrixMarket matrix coordinate real general\n3 3 1\n4 1 1\n",  # row out of range
    "%%MatrixMarket matrix coordinate real general\n3 3 1\n0 1 1\n",  # 0 in a 1-based file
    "%%MatrixMarket matrix coordinate real general\n3 3 1\n1 x 1\n",  # malformed
])
def test_read_mtx_rejects_bad_files(tmp_path, text):
    p = tmp_path / "bad.mtx"
    p.write_text(text)
    with pytest.raises(E.AesError) as ei:
        E.read_mtx(str(p))
    assert ei.value.code in (E.AES_ERR_INVALID, E.AES_ERR_UNSUPPORTED)


def test_read_mtx_feeds_create_path(tmp_path):
    """A file written from a generated CSR reads back to the same CSR once sorted."""
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, 2000, 300, 3, 9, seed=8)
    row = np.repeat(np.arange(2000, dtype=np.uint32), np.diff(ptr).astype(np.int64))
    perm = np.random.default_rng(1).permutation(len(col))
    p = str(tmp_path / "g.mtx")
    E.write_mtx(p, 2000, 300, row[perm], col[perm], val[perm])
    rows, cols, r, c, v = E.read_mtx(p, E.MTX_SORT)
    assert np.array_equal(r, row) and np.array_equal(c, col)
    assert np.array_equal(_bits(v), _bits(val))


# ---- ReSparse ---------------------------------------------------------------------------------

def _resparse_cases():
    g = np.load(os.path.join(GOLD, "resparse.npz"))
    out = []
    i = 0
    while f"m{i}_shape" in g.files:
        for j, keep in enumerate(g[f"m{i}_keeps"]):
            out.append((i, j, float(keep)))
        i += 1
    return g, out


_RG, _RCASES = _resparse_cases()


@pytest.mark.parametrize("impl", ["oracle", "library"])
@pytest.mark.parametrize("case", _RCASES, ids=[f"m{i}-keep{k}" for i, _, k in _RCASES])
def test_resparse_matches_reference_golden(impl, case):
    i, j, keep = case
    g = _RG
    rows, cols = (int(x) for x in g[f"m{i}_shape"])
    fn = orc.resparse if impl == "oracle" else E.resparse
    p, c, v = fn(g[f"m{i}_ptr"], g[f"m{i}_col"], g[f"m{i}_val"], rows, cols, keep)
    assert np.array_equal(p, g[f"m{i}_k{j}_ptr"])
    assert np.array_equal(c, g[f"m{i}_k{j}_col"])
    assert np.array_equal(_bits(v), _bits(g[f"m{i}_k{j}_val"]))


@pytest.mark.parametrize("keep", [0.999, 0.776, 0.5, 0.3, 0.01])
def test_resparse_library_matches_oracle(keep):
    """Larger seeded inputs with explicit zeros, empty rows and equal magnitudes across the cut
    (the documented rule: higher column first)."""
    rng = np.random.default_rng(int(keep * 1000))
    rows, cols = 3000, 200
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, rows, cols, 0, 40, seed=3)
    val = val.copy()
    val[rng.random(len(val)) < 0.05] = 0.0
    sel = rng.random(len(val)) < 0.3
    val[sel] = np.round(val[sel] * 4) / 4 * np.where(rng.random(sel.sum()) < 0.5, -1, 1)
    a = E.resparse(ptr, col, val, rows, cols, keep)
    b = orc.resparse(ptr, col, val, rows, cols, keep)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(_bits(a[2]), _bits(b[2]))


def test_resparse_rejects_bad_input():
    ptr = np.array([0, 2], np.uint64)
    with pytest.raises(E.AesError):
        E.resparse(ptr, np.array([3, 3], np.uint32), np.ones(2, np.float32), 1, 8, 0.5)
    with pytest.raises(E.AesError):
        E.resparse(ptr, np.array([1, 3], np.uint32), np.ones(2, np.float32), 1, 8, 0.0)
    with pytest.raises(E.AesError):
        E.resparse(ptr, np.array([1, 3], np.uint32), np.ones(2, np.float32), 1, 8, 1.5)


# ---- keep-ratio search ------------------------------------------------------------------------

@pytest.mark.parametrize("knee", [0.0, 0.13, 0.5, 0.777, 0.9991, 1.0])
@pytest.mark.parametrize("thr", [0.999, 0.9])
def test_bisect_keep_follows_reference_loop(knee, thr):
    """Same ratios tried, same answer as the oracle's restatement of the reference loop, on
    metrics that fall off below a knee."""
    def metric(keep, epoch):
        return 1.0 if keep >= knee else keep / max(knee, 1e-9) * 0.9

    a = RS.bisect_keep(metric, thr)
    b = orc.search_keep_ratio(metric, thr)
    assert a[0] == b[0]
    assert [h[:2] for h in a[1]] == [h[:2] for h in b[1]]


def test_precision_metric_matches_oracle():
    rng = np.random.default_rng(2)
    precs_a, precs_b = [], []
    for _ in range(7):
        exact = rng.permutation(500)[:100]
        cand = rng.permutation(500)[:256]
        precs_a.append(RS.precision_at(exact, cand))
        precs_b.append(orc.compt_precision(exact, cand))
    assert precs_a == precs_b
    assert RS.epoch_metric(precs_a) == pytest.approx(orc.convergence_metric(precs_b), rel=0, abs=1e-15)
