"""The C++ drop-in (include/acceles_spmv.hpp) compiles against the library, and on a GPU a
main() in the reference's call order returns the oracle's results."""
import os
import subprocess

import numpy as np
import pytest

import oracle as orc
from acceles_gb300 import engine as E, _build

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
EXE = os.path.join(REPO, "acceles_gb300", "_lib", "spmv_api_main")


def build_exe():
    E.load()
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(REPO, "include"),
                    os.path.join(HERE, "cpp", "spmv_api_main.cpp"), "-o", EXE,
                    "-L", os.path.dirname(_build.LIB), "-lacceles",
                    "-Wl,-rpath," + os.path.dirname(_build.LIB)], check=True)
    return EXE


def test_cpp_wrapper_compiles_and_links():
    assert os.path.exists(build_exe())


@pytest.mark.gpu
def test_cpp_wrapper_matches_oracle():
    res = subprocess.run([build_exe(), "7"], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    out = res.stdout
    lines = {l.split(" ", 1)[0]: l.split(" ", 1)[1] for l in out.strip().splitlines()}
    q = np.array([float(v) for v in lines["query"].split()], np.float32)
    cand = [tuple(t.split(":")) for t in lines["cand"].split()]
    top = [tuple(t.split(":")) for t in lines["top"].split()]
    rows, cols = 30000, 512
    ptr, col, val = E.gen_matrix(E.GEN_UNIFORM_DEG, rows, cols, 10, 30, seed=7)
    m = orc.Matrix(rows, cols, ptr, col, val, 6, orc.QUANT_SYM_GLOBAL)
    oi, os_, oc = m.two_stage(q, 32, 512, 100)
    assert [int(i) for i, _ in top] == list(oi)
    assert np.array_equal(np.array([float(s) for _, s in top], np.float32), os_)
    keys = m.keys(q)
    exp = oc[np.lexsort((-oc.astype(np.int64), -keys[oc].astype(np.int64)))]
    assert [int(i) for i, _ in cand] == list(exp)
    assert all(int(s) == int(keys[int(i)]) - (1 << 31) for i, s in cand)
