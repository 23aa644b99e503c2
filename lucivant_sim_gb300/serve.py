"""Serving: a continuous-batching request loop on one GPU.

Jobs arrive as OpenQASM text at any time (:meth:`Server.submit` returns a future). A job is
prepared on the host in a pool of spawned processes (parsing, operator lists — Python host work
that would otherwise serialise on the interpreter lock), then admitted to the device as soon as a
worker slot and its device memory (2^n or 4^n amplitudes x bytes per amplitude, times the sweep
size) are free. Admitted jobs run concurrently: every worker owns its registers, each with its own
CUDA stream, so the passes of different jobs overlap on the device, and a finishing job's memory
and slot go to the next waiting job immediately — no batch boundary. A parameter sweep is one
batched register (one member per parameter set, per-member gate data), so its points share every
pass.

Job kinds (dicts, as :func:`lucivant_sim_gb300.workloads.served_mix` makes them):

* ``sample``: statevector, ``shots`` samples with Orrery's draw order and ``seed``;
* ``expect``: a parameter sweep of one ``input``-parameterised template, the expectation of a
  weighted Pauli sum for every parameter set;
* ``density``: noisy density matrix (uniform noise), ``shots`` samples with readout error.

Results do not depend on what else runs: every job's arithmetic is the same kernels on its own
register, so a job's result alone and in the mix is identical (checked by ``tests``).
"""

from __future__ import annotations

import heapq
import multiprocessing as mp
import os
import threading
import time
from concurrent.futures import Future, ProcessPoolExecutor
from dataclasses import dataclass, field
from typing import Any

import numpy as np

from lucivant_sim_gb300 import _lib, engine
from lucivant_sim_gb300.noise import NoiseModel
from lucivant_sim_gb300.simulator import sample_register

DEFAULT_NOISE = dict(single=1e-3, two=1e-2, readout=2e-2)


# --------------------------------------------------------------------------- host preparation


def prepare(job: dict) -> dict:
    """Host side of a job: parse, build the device operator list (runs in a worker process)."""
    from lucivant_sim_gb300 import qasm

    kind = job["kind"]
    out: dict[str, Any] = {"kind": kind, "id": job.get("id")}
    if kind == "sample":
        c = qasm.parse(job["qasm"])
        out.update(nbits=c.num_qubits, batch=1, ops=engine.sv_oplist(c).packed(), circuit=c, noise=None,
                   shots=job["shots"], seed=job["seed"], dm=0)  # fmt: skip
    elif kind == "density":
        c = qasm.parse(job["qasm"])
        noise = job.get("noise", DEFAULT_NOISE)
        models = [NoiseModel.uniform(**noise)]
        real = engine.dm_form(c, models) == "ptm"
        ops = engine.ptm_oplist(c, models) if real else engine.dm_oplist(c, models)
        out.update(nbits=2 * c.num_qubits, batch=1, ops=ops.packed(), circuit=c, noise=noise, real=real,
                   shots=job["shots"], seed=job["seed"], dm=c.num_qubits)  # fmt: skip
    elif kind == "expect":
        circuits = [qasm.parse(job["qasm"], p) for p in job["params"]]
        out.update(nbits=circuits[0].num_qubits, batch=len(circuits), ops=sweep_oplist(circuits).packed())
        labels = list(job["observable"])
        masks = [engine.pauli_masks(lab) for lab in labels]
        out.update(xmask=[m[0] for m in masks], zmask=[m[1] for m in masks],
                   weights=[float(job["observable"][lab]) for lab in labels])  # fmt: skip
    else:
        raise ValueError(f"unknown job kind {kind!r}")
    return out


def sweep_oplist(circuits: list[Any]) -> _lib.OpList:
    """One batched operator list for circuits of the same structure (a parameter sweep): each
    gate position carries one matrix per member."""
    seqs = [engine.fuse_runs(c.operations) for c in circuits]
    ops = _lib.OpList()
    for pos, first in enumerate(seqs[0]):
        if first.kind != "gate":
            continue
        mats = [np.asarray(s[pos].matrix, dtype=np.complex128) for s in seqs]
        kinds = {engine.classify(m)[0] for m in mats}
        kind, datas = _lib.OP_MATRIX, mats  # mixed classes across the sweep: dense for all
        if len(kinds) == 1:
            kind = kinds.pop()
            datas = [engine.classify(m)[1] for m in mats]
        same = all(np.array_equal(datas[0], d) for d in datas[1:])
        if kind == _lib.OP_PERM and not same:  # permutations are planned from member 0's table
            kind, datas = _lib.OP_MATRIX, mats
        if same:
            ops.add(kind, list(first.qubits), datas[0])
        else:
            ops.add_batched(kind, list(first.qubits), np.stack(datas))
    return ops


# --------------------------------------------------------------------------- device workers


class _RegisterPool:
    """Registers kept for reuse by shape: allocation stays off the serving path."""

    def __init__(self) -> None:
        self.free: dict[tuple[int, int, int], list[_lib.Register]] = {}
        self.lock = threading.Lock()

    def take(self, nbits: int, precision: int, batch: int) -> _lib.Register:
        with self.lock:
            lst = self.free.get((nbits, precision, batch))
            if lst:
                return lst.pop()
        return _lib.Register(nbits, precision, batch)

    def give(self, reg: _lib.Register) -> None:
        with self.lock:
            self.free.setdefault((reg.nbits, reg.precision, reg.batch), []).append(reg)

    def clear(self) -> None:
        with self.lock:
            for lst in self.free.values():
                for r in lst:
                    r.free()
            self.free.clear()


def execute(prep: dict, precision: int, pool: _RegisterPool | None = None) -> dict:
    """Device side of a prepared job (runs on a server worker thread, or alone)."""
    nbits, batch = prep["nbits"], prep["batch"]
    if prep.get("real"):  # a density matrix in Pauli-transfer form
        precision = engine.REAL_OF[precision]
    reg = pool.take(nbits, precision, batch) if pool else _lib.Register(nbits, precision, batch)
    try:
        table, flat = prep["ops"]  # |0...0> then the operators (tiles not reached yet are skipped)
        _lib.check(reg.lib.lsg_apply_from_basis(reg.handle, 0, table.ctypes.data, len(table),
                                                _lib.ptr(flat, _lib.C.c_double), flat.size // 2))  # fmt: skip
        if prep["kind"] == "expect":
            vals = reg.expect(0, prep["xmask"], prep["zmask"])  # (terms, batch)
            w = np.asarray(prep["weights"])
            return {"values": (w[:, None] * vals).sum(axis=0)}
        noise = NoiseModel.uniform(**prep["noise"]) if prep["noise"] else None
        counts, report = sample_register(reg, prep["circuit"], prep["dm"], prep["shots"], noise,
                                         np.random.default_rng(prep["seed"]))  # fmt: skip
        return {"counts": counts, "near_boundary": report["near_boundary"]}
    finally:
        if pool:
            pool.give(reg)
        else:
            reg.free()


def job_bytes(prep: dict, precision: int) -> int:
    elt = _lib.ELEM_BYTES[engine.REAL_OF[precision] if prep.get("real") else precision]
    return (elt << prep["nbits"]) * prep["batch"] * 2 + (64 << 20)  # register, reductions, program


@dataclass(order=True)
class _Waiting:
    order: int
    prep: dict = field(compare=False)
    future: Future = field(compare=False)
    need: int = field(compare=False)


class Server:
    """Continuous-batching server: submit jobs, get futures."""

    def __init__(self, precision: str = "c64", workers: int = 8, prep_workers: int | None = None,
                 memory_fraction: float = 0.6, memory_bytes: int | None = None) -> None:  # fmt: skip
        _lib.ensure_device()
        self.precision = engine.precision_code(precision)
        free, _total = _lib.mem_info()
        self.budget = int(memory_bytes if memory_bytes is not None else free * memory_fraction)
        self.used = 0
        self.slots = workers
        self.pool = _RegisterPool()
        self.cv = threading.Condition()
        self.waiting: list[_Waiting] = []
        self.counter = 0
        self.closed = False
        self.device = _lib._default_device
        nprep = prep_workers or max(1, min(16, (os.cpu_count() or 2) - 1))
        self.prep = ProcessPoolExecutor(max_workers=nprep, mp_context=mp.get_context("spawn"))
        self.threads = [threading.Thread(target=self._worker, daemon=True) for _ in range(workers)]
        for t in self.threads:
            t.start()

    # -- client side ---------------------------------------------------------------------
    def submit(self, job: dict) -> Future:
        """Queue a job; the future resolves to its result dict (plus ``latency_s``)."""
        fut: Future = Future()
        t0 = time.perf_counter()
        pf = self.prep.submit(prepare, job)
        pf.add_done_callback(lambda f: self._prepared(f, fut, t0))
        return fut

    def _prepared(self, pf: Any, fut: Future, t0: float) -> None:
        try:
            prep = pf.result()
        except Exception as exc:  # noqa: BLE001 - handed to the client
            fut.set_exception(exc)
            return
        prep["t0"] = t0
        need = job_bytes(prep, self.precision)
        if need > self.budget:
            fut.set_exception(MemoryError(f"the job needs {need} bytes; the server admits at most {self.budget}"))
            return
        with self.cv:
            self.counter += 1
            heapq.heappush(self.waiting, _Waiting(self.counter, prep, fut, need))
            self.cv.notify()

    # -- device side ---------------------------------------------------------------------
    def _admit(self) -> _Waiting | None:
        """The oldest waiting job that fits the free memory (oldest first; a smaller job may pass a
        big one that does not fit yet)."""
        for i, w in enumerate(sorted(self.waiting)):
            if self.used + w.need <= self.budget:
                self.waiting.remove(w)
                heapq.heapify(self.waiting)
                self.used += w.need
                return w
        return None

    def _worker(self) -> None:
        _lib.ensure_device(self.device)
        while True:
            with self.cv:
                w = None
                while not self.closed:
                    w = self._admit() if self.waiting else None
                    if w is not None:
                        break
                    self.cv.wait(0.05)
                if w is None:
                    return
            try:
                res = execute(w.prep, self.precision, self.pool)
                res["latency_s"] = time.perf_counter() - w.prep["t0"]
                w.future.set_result(res)
            except Exception as exc:  # noqa: BLE001 - handed to the client
                w.future.set_exception(exc)
            finally:
                with self.cv:
                    self.used -= w.need
                    self.cv.notify_all()

    def close(self) -> None:
        with self.cv:
            self.closed = True
            self.cv.notify_all()
        for t in self.threads:
            t.join(timeout=60)
        self.prep.shutdown(wait=True, cancel_futures=True)
        self.pool.clear()

    def __enter__(self) -> Server:
        return self

    def __exit__(self, *exc: Any) -> None:
        self.close()


def replay(jobs: list[dict], server: Server, realtime: bool = True) -> dict:
    """Submit ``jobs`` at their arrival times (or all at once) and wait: results in job order,
    p50/p99 latency and throughput."""
    start = time.perf_counter()
    futures = []
    for i, job in enumerate(jobs):
        job = dict(job, id=i)
        if realtime:
            delay = start + job["arrival"] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
        futures.append(server.submit(job))
    results = [f.result() for f in futures]
    elapsed = time.perf_counter() - start
    lat = np.array([r["latency_s"] for r in results])
    return {
        "results": results,
        "elapsed_s": elapsed,
        "circuits_per_s": len(jobs) / elapsed,
        "p50_s": float(np.percentile(lat, 50)),
        "p99_s": float(np.percentile(lat, 99)),
    }
