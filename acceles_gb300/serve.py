"""Serving loop: several device-resident matrices, continuous batching, admission by memory.

Each matrix is resident once and has one or more batch slots: the engine handle that owns it and
views of it (aes_create_view), each with its own CUDA stream and batch buffers, each served by
one worker thread.  A request (matrix, FP32 query, K) is queued on its matrix; a free slot's
worker takes every request waiting (up to max_batch), runs them as one batch (from 16 queries on,
one matrix read scores 128 queries) and completes each request with its first K results.
Requests that arrive while batches are on the GPU join the next batch as soon as a slot frees;
batches of one matrix, and of different matrices, run on the GPU at the same time.

Admission by device memory: a matrix is admitted only if the matrix and one batch slot fit the
server's budget (the handle's mem_limit makes creation fail before allocating); each further
slot is admitted only while its batch buffers still fit.

Results do not depend on batching: each request's Top-K is the same alone and in any mix.

  python -m acceles_gb300.serve [--rates 1000,10000,50000] [--duration 5] [--small]
"""
from __future__ import annotations

import argparse
import json
import queue
import threading
import time
from concurrent.futures import Future

import numpy as np

from . import engine as E


class _Request:
    __slots__ = ("query", "k", "future", "t_submit")

    def __init__(self, query, k):
        self.query = query
        self.k = k
        self.future = Future()
        self.t_submit = time.perf_counter()


class _Matrix:
    def __init__(self, name, engines, cols, max_batch, k_max):
        self.name = name
        self.slots = engines  # the owning handle first, then its views
        self.cols = cols
        self.max_batch = max_batch
        self.k_max = k_max
        self.q = queue.Queue()
        self.threads = []
        self.batches = 0
        self.served = 0
        self.lock = threading.Lock()
        self.in_flight = 0      # batches of this matrix on the GPU now
        self.max_in_flight = 0  # the most at once so far


class Server:
    """Top-K SpMV server over device-resident matrices."""

    def __init__(self, device: int = 0, mem_budget: int | None = None, slots: int = 2):
        self.device = device
        self.mem_budget = mem_budget
        self.slots = slots
        self.mem_used = 0
        self.mats: dict[str, _Matrix] = {}
        self.running = False
        self.lock = threading.Lock()

    # ---- admission ---------------------------------------------------------------------------
    def _limit(self):
        if self.mem_budget is None:
            return 0
        return max(1, self.mem_budget - self.mem_used)

    def add_matrix(self, name, rows, cols, ptr, col, val, max_batch=256, k_max=100, slots=None,
                   **params):
        """Create a resident matrix with up to `slots` batch slots (the server's default if
        None); raises AesError(AES_ERR_NOMEM) if the matrix and one slot do not fit.  Returns
        the owning handle's info with the number of slots admitted."""
        with self.lock:
            eng = E.SpMV(rows, cols, ptr=ptr, col=col, val=val, max_batch=max_batch,
                         k_max=k_max, device=self.device, mem_limit=self._limit(),
                         flags=params.pop("flags", E.FLAG_GRAPHS), **params)
            self.mem_used += eng.info()["device_bytes"]
            engines = [eng]
            for _ in range((slots or self.slots) - 1):
                try:
                    v = eng.view(mem_limit=self._limit())
                except E.AesError as ex:
                    if ex.code != E.AES_ERR_NOMEM:
                        raise
                    break  # the next slot's batch buffers do not fit the budget
                self.mem_used += v.info()["device_bytes"]
                engines.append(v)
            m = _Matrix(name, engines, cols, max_batch, k_max)
            self.mats[name] = m
            if self.running:
                self._start_workers(m)
            info = eng.info()
            info["slots"] = len(engines)
            return info

    # ---- requests ----------------------------------------------------------------------------
    def submit(self, name, query, k) -> Future:
        m = self.mats[name]
        if k > m.k_max:
            raise ValueError("k above the matrix's k_max")
        r = _Request(np.ascontiguousarray(query, np.float32), int(k))
        m.q.put(r)
        return r.future

    # ---- workers -----------------------------------------------------------------------------
    def start(self):
        self.running = True
        for m in self.mats.values():
            self._start_workers(m)

    def stop(self):
        self.running = False
        for m in self.mats.values():
            for _ in m.threads:
                m.q.put(None)
        for m in self.mats.values():
            for t in m.threads:
                t.join()
            m.threads = []

    def _start_workers(self, m):
        for eng in m.slots:
            t = threading.Thread(target=self._worker, args=(m, eng), daemon=True)
            t.start()
            m.threads.append(t)

    def _worker(self, m: _Matrix, eng):
        buf = np.zeros((m.max_batch, m.cols), np.float32)
        while True:
            first = m.q.get()
            if first is None:
                return
            batch = [first]
            while len(batch) < m.max_batch:  # everything that arrived meanwhile joins
                try:
                    r = m.q.get_nowait()
                except queue.Empty:
                    break
                if r is None:
                    m.q.put(None)
                    break
                batch.append(r)
            n = len(batch)
            kmax = max(r.k for r in batch)
            for i, r in enumerate(batch):
                buf[i] = r.query
            with m.lock:
                m.in_flight += 1
                m.max_in_flight = max(m.max_in_flight, m.in_flight)
            try:
                eng.Q_reset(buf[:n])
                eng(k=kmax)  # the GIL is released while the slot's stream runs
                idx, sc = eng.read_topk()
            except Exception as ex:  # report the failure to every request of the batch
                for r in batch:
                    r.future.set_exception(ex)
                continue
            finally:
                with m.lock:
                    m.in_flight -= 1
            t = time.perf_counter()
            for i, r in enumerate(batch):
                r.future.set_result((idx[i, :r.k].copy(), sc[i, :r.k].copy(), t - r.t_submit))
            with m.lock:
                m.batches += 1
                m.served += n

    def close(self):
        self.stop()
        for m in self.mats.values():
            for eng in reversed(m.slots):
                eng.close()
        self.mats.clear()


def run_load(server: Server, names, cols_of, rate, duration, ks=(8, 32, 100), seed=0):
    """Poisson arrivals at `rate` queries/s for `duration` s; each request picks a matrix and K
    uniformly.  Returns (throughput, p50, p99, completed)."""
    rng = np.random.default_rng(seed)
    futures = []
    t0 = time.perf_counter()
    t_next = t0
    qcache = {n: rng.random((64, cols_of[n])).astype(np.float32) for n in names}
    i = 0
    while True:
        t_next += rng.exponential(1.0 / rate)
        if t_next - t0 > duration:
            break
        now = time.perf_counter()
        if t_next > now:
            time.sleep(t_next - now)
        n = names[int(rng.integers(len(names)))]
        k = int(ks[int(rng.integers(len(ks)))])
        futures.append(server.submit(n, qcache[n][i % 64], k))
        i += 1
    lat = np.array([f.result()[2] for f in futures])
    t_end = time.perf_counter()
    return len(futures) / (t_end - t0), float(np.percentile(lat, 50)), float(np.percentile(lat, 99)), len(futures)


def serving_specs(scale=1):
    """The three resident matrices of the serving workload: (name, generator, rows, cols, p0,
    p1, seed); 1/scale of the rows for a small run."""
    return [
        ("1Mx900_12pct", E.GEN_FIXED_UNIFORM, 1_000_000 // scale, 900, 108, 0, 5101),
        ("10Mx1024_deg20", E.GEN_UNIFORM_DEG, 10_000_000 // scale, 1024, 10, 30, 5102),
        ("20Mx512_gamma32", E.GEN_GAMMA_DEG, 20_000_000 // scale, 512, 32, 512, 5103),
    ]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--rates", default="1000,10000,50000")
    ap.add_argument("--duration", type=float, default=5.0)
    ap.add_argument("--small", action="store_true", help="1/10 sized matrices")
    ap.add_argument("--max-batch", type=int, default=256)
    ap.add_argument("--slots", type=int, default=2, help="batch slots per matrix")
    args = ap.parse_args()
    s = 10 if args.small else 1
    srv = Server(slots=args.slots)
    cols_of = {}
    for name, kind, rows, cols, p0, p1, seed in serving_specs(s):
        ptr, col, val = E.gen_matrix(kind, rows, cols, p0, p1, seed=seed)
        info = srv.add_matrix(name, rows, cols, ptr, col, val, max_batch=args.max_batch,
                              k_max=100, bits=8, split=1, ck=1024, flags=0)
        cols_of[name] = cols
        print(json.dumps({"matrix": name, "rows": rows, "nnz": info["nnz"],
                          "device_bytes": info["device_bytes"], "slots": info["slots"]}),
              flush=True)
    srv.start()
    names = [sp[0] for sp in serving_specs(s)]
    run_load(srv, names, cols_of, 200, 1.0, seed=99)  # warm-up: graphs, caches
    for rate in [float(r) for r in args.rates.split(",")]:
        qps, p50, p99, n = run_load(srv, names, cols_of, rate, args.duration, seed=int(rate))
        print(json.dumps({"offered_qps": rate, "served_qps": qps, "p50_ms": p50 * 1e3,
                          "p99_ms": p99 * 1e3, "requests": n,
                          "batches": {m.name: m.batches for m in srv.mats.values()},
                          "max_in_flight": {m.name: m.max_in_flight for m in srv.mats.values()}}),
              flush=True)
    srv.close()


if __name__ == "__main__":
    main()
