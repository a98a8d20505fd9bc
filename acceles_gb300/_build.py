"""Build the engine's shared library in-tree: acceles_gb300/_lib/libacceles.so.

nvcc compiles the CUDA translation units for sm_103a only; the host C++ compiles with the
system g++.  Units compile in parallel; nothing is rebuilt when its inputs are unchanged.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(REPO, "include")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libacceles.so")
# the library-SpMV comparison arm lives in its own library so that the engine does not load
# cuSPARSE: its CUDA unit plus the host helpers it shares with the engine
BASELINE_LIB = os.path.join(OUT_DIR, "libaes_baseline.so")
BASELINE_ONLY = ("aes_gpu_baseline.cu",)
BASELINE_SHARED = ("aes_host.cpp",)

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [GENCODE, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
              "-diag-suppress", "177"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-pthread"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _digest(paths, extra: str) -> str:
    h = hashlib.sha256(extra.encode())
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    cu, cpp = _sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    hdr_digest = _digest(sorted(headers), "hdr")
    nvcc = _nvcc()
    objs = []
    obj_of = {}
    jobs = []
    for f in cu + cpp:
        src = os.path.join(CSRC, f)
        is_cu = f.endswith(".cu")
        flags = NVCC_FLAGS if is_cu else CXX_FLAGS
        key = _digest([src], hdr_digest + " ".join(flags) + sys.platform + os.uname().machine)
        obj = os.path.join(OUT_DIR, f"{f}.{key}.o")
        objs.append(obj)
        obj_of[f] = obj
        if os.path.exists(obj) and not force:
            continue
        if is_cu:
            cmd = [nvcc] + flags + ["-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
        else:
            cmd = ["g++"] + flags + ["-I", INCLUDE, "-I", CSRC,
                                    "-I", os.path.join(_cuda_home(), "include"), "-c", src, "-o", obj]
        jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    eng_objs = [obj_of[f] for f in cu + cpp if f not in BASELINE_ONLY]
    base_objs = [obj_of[f] for f in BASELINE_ONLY + BASELINE_SHARED if f in obj_of]
    _link(nvcc, LIB, eng_objs, ["-lcudart", "-lpthread"], force, run)
    _link(nvcc, BASELINE_LIB, base_objs, ["-lcusparse", "-lcudart", "-lpthread"], force, run)
    # drop objects of older source versions
    keep = set(os.path.basename(o) for o in objs)
    for f in os.listdir(OUT_DIR):
        if f.endswith(".o") and f not in keep:
            os.remove(os.path.join(OUT_DIR, f))
    return LIB


def _link(nvcc, lib, objs, libs, force, run):
    link_key = _digest(objs, "link " + " ".join(libs))
    stamp = lib + ".stamp"
    if os.path.exists(lib) and os.path.exists(stamp) and open(stamp).read() == link_key and not force:
        return
    tmp = lib + ".tmp"
    run([nvcc, GENCODE, "-shared", "-o", tmp] + objs + libs)
    os.replace(tmp, lib)
    with open(stamp, "w") as f:
        f.write(link_key)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
