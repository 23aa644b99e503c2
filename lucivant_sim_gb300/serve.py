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

import hashlib
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
    if kind in ("sample", "density"):
        out["key"] = structure_key(out)
    return out


def structure_key(prep: dict) -> str:
    """Jobs with equal keys can share one register: the same kind, register and operator
    structure (kinds, bits, data sizes), whatever the operators' values."""
    table, flat = prep["ops"]
    h = hashlib.sha1()
    h.update(f"{prep['kind']}:{prep['nbits']}:{prep.get('real', False)}:{flat.size}:".encode())
    h.update(table.tobytes())
    return h.hexdigest()


def combined_ops(preps: list[dict]) -> tuple[np.ndarray, np.ndarray]:
    """One operator table for jobs of one structure key, member b = job b: operators whose data
    agree across the jobs keep one copy, the others carry one copy per member."""
    table = preps[0]["ops"][0]
    pools = np.stack([p["ops"][1].view(np.complex128) for p in preps])  # (members, entries)
    starts = table["data"].astype(np.int64)
    order = np.argsort(starts, kind="stable")
    ends = np.empty_like(starts)
    ends[order[:-1]] = starts[order[1:]]
    ends[order[-1]] = pools.shape[1]
    out = table.copy()
    chunks, at = [], 0
    for i in range(len(table)):
        seg = pools[:, starts[i]:ends[i]]
        if (seg == seg[0]).all():
            chunks.append(seg[0])
            out[i]["data"], out[i]["batch_stride"] = at, 0
            at += seg.shape[1]
        else:
            chunks.append(seg.reshape(-1))
            out[i]["data"], out[i]["batch_stride"] = at, seg.shape[1]
            at += seg.size
    flat = np.concatenate(chunks) if chunks else np.zeros(1, dtype=np.complex128)
    return out, np.ascontiguousarray(flat.view(np.float64))


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
    """Idle registers kept for reuse by shape: allocation stays off the serving path. Their
    device bytes (``bytes``) stay allocated, so the server counts them against its budget and
    frees idle registers when an admission needs the room."""

    def __init__(self) -> None:
        self.free: dict[tuple[int, int, int], list[_lib.Register]] = {}
        self.bytes = 0
        self.lock = threading.Lock()

    def take(self, shape: tuple[int, int, int]) -> _lib.Register | None:
        """An idle register of ``shape`` (nbits, precision, batch), or None."""
        with self.lock:
            lst = self.free.get(shape)
            if not lst:
                return None
            reg = lst.pop()
            self.bytes -= register_bytes(*shape)
            return reg

    def give(self, reg: _lib.Register) -> None:
        with self.lock:
            self.free.setdefault((reg.nbits, reg.precision, reg.batch), []).append(reg)
            self.bytes += register_bytes(reg.nbits, reg.precision, reg.batch)

    def evict(self, nbytes: int) -> int:
        """Free idle registers, largest first, until at least ``nbytes`` are released (or none are
        left); returns the bytes released."""
        with self.lock:
            regs = sorted((r for lst in self.free.values() for r in lst),
                          key=lambda r: register_bytes(r.nbits, r.precision, r.batch), reverse=True)  # fmt: skip
            released = 0
            for r in regs:
                if released >= nbytes:
                    break
                self.free[(r.nbits, r.precision, r.batch)].remove(r)
                size = register_bytes(r.nbits, r.precision, r.batch)
                r.free()
                released += size
                self.bytes -= size
            self.free = {k: v for k, v in self.free.items() if v}
            return released

    def clear(self) -> int:
        return self.evict(self.bytes + 1)


def register_bytes(nbits: int, precision: int, batch: int) -> int:
    return (_lib.ELEM_BYTES[precision] << nbits) * batch


def execute(prep: dict, precision: int, reg: _lib.Register | None = None) -> dict:
    """Device side of a prepared job (runs on a server worker thread, or alone). ``reg``: a
    register of the job's shape to run on (kept by the caller), else one is made and freed."""
    nbits, batch = prep["nbits"], prep["batch"]
    precision = job_precision(prep, precision)
    own = reg is None
    if own:
        reg = _lib.Register(nbits, precision, batch)
    try:
        t0 = time.perf_counter()
        table, flat = prep["ops"]  # |0...0> then the operators (tiles not reached yet are skipped)
        _lib.check(reg.lib.lsg_apply_from_basis(reg.handle, 0, table.ctypes.data, len(table),
                                                _lib.ptr(flat, _lib.C.c_double), flat.size // 2))  # fmt: skip
        t1 = time.perf_counter()  # planning, upload and the passes (the call waits for them)
        if prep["kind"] == "expect":
            vals = reg.expect(0, prep["xmask"], prep["zmask"])  # (terms, batch)
            w = np.asarray(prep["weights"])
            return {"values": (w[:, None] * vals).sum(axis=0), "apply_s": t1 - t0,
                    "reduce_s": time.perf_counter() - t1}  # fmt: skip
        noise = NoiseModel.uniform(**prep["noise"]) if prep["noise"] else None
        counts, report = sample_register(reg, prep["circuit"], prep["dm"], prep["shots"], noise,
                                         np.random.default_rng(prep["seed"]))  # fmt: skip
        return {"counts": counts, "near_boundary": report["near_boundary"], "apply_s": t1 - t0,
                "reduce_s": time.perf_counter() - t1}  # fmt: skip
    finally:
        if own:
            reg.free()


def execute_group(preps: list[dict], precision: int, reg: _lib.Register | None = None) -> list[dict]:
    """Jobs of one structure key on one register (member b = job b): one program, one launch per
    pass for all of them, then each member sampled with its own seed and noise. Each member's
    arithmetic is the same as alone (the same operators, per-member data), so each result is the
    job's result alone."""
    if len(preps) == 1:
        return [execute(preps[0], precision, reg)]
    first = preps[0]
    code = job_precision(first, precision)
    own = reg is None
    if own:
        reg = _lib.Register(first["nbits"], code, len(preps))
    try:
        table, flat = combined_ops(preps)
        _lib.check(reg.lib.lsg_apply_from_basis(reg.handle, 0, table.ctypes.data, len(table),
                                                _lib.ptr(flat, _lib.C.c_double), flat.size // 2))  # fmt: skip
        out = []
        for b, prep in enumerate(preps):
            noise = NoiseModel.uniform(**prep["noise"]) if prep["noise"] else None
            counts, report = sample_register(reg, prep["circuit"], prep["dm"], prep["shots"], noise,
                                             np.random.default_rng(prep["seed"]), member=b)  # fmt: skip
            out.append({"counts": counts, "near_boundary": report["near_boundary"], "batched_with": len(preps)})
        return out
    finally:
        if own:
            reg.free()


def job_precision(prep: dict, precision: int) -> int:
    """The register precision of a job: density matrices in Pauli-transfer form are real."""
    return engine.REAL_OF[precision] if prep.get("real") else precision


def job_shape(prep: dict, precision: int) -> tuple[int, int, int]:
    return prep["nbits"], job_precision(prep, precision), prep["batch"]


def group_shape(group: list[Any], precision: int) -> tuple[int, int, int]:
    """The register of a group of waiting jobs of one structure key: one member per job (a
    sweep's members when alone)."""
    nbits, code, batch = job_shape(group[0].prep, precision)
    return nbits, code, batch if len(group) == 1 else len(group)


def job_bytes(prep: dict, precision: int) -> int:
    """Device bytes a job holds while it runs: its register, as much again for reductions, and
    room for the program."""
    return 2 * register_bytes(*job_shape(prep, precision)) + (64 << 20)


@dataclass(order=True)
class _Waiting:
    order: int
    prep: dict = field(compare=False)
    future: Future = field(compare=False)
    need: int = field(compare=False)


class Server:
    """Continuous-batching server: submit jobs, get futures."""

    def __init__(self, precision: str = "c64", workers: int = 16, prep_workers: int | None = None,
                 memory_fraction: float = 0.6, memory_bytes: int | None = None, group_max: int = 16) -> None:  # fmt: skip
        _lib.ensure_device()
        self.precision = engine.precision_code(precision)
        free, _total = _lib.mem_info()
        self.budget = int(memory_bytes if memory_bytes is not None else free * memory_fraction)
        self.used = 0
        self.slots = workers
        self.group_max = max(1, int(group_max))  # jobs of one structure key run together, up to this many
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
        except Exception as exc:  # noqa: BLE001 - handed to the client (a cancelled preparation too)
            fut.set_exception(RuntimeError("server closed") if pf.cancelled() else exc)
            return
        prep["t0"] = t0
        prep["t_prepared"] = time.perf_counter()
        need = job_bytes(prep, self.precision)
        if need > self.budget:
            fut.set_exception(MemoryError(f"the job needs {need} bytes; the server admits at most {self.budget}"))
            return
        with self.cv:
            if self.closed:
                fut.set_exception(RuntimeError("server closed"))
                return
            self.counter += 1
            heapq.heappush(self.waiting, _Waiting(self.counter, prep, fut, need))
            self.cv.notify()

    # -- device side ---------------------------------------------------------------------
    # ``used`` counts the full need of every running job plus the idle pooled registers (they stay
    # allocated). A job that reuses an idle register of its shape needs only the rest of its need.
    def _admit(self) -> tuple[list[_Waiting], _lib.Register | None] | None:
        """The oldest waiting job that fits the free memory (oldest first; a smaller job may pass a
        big one that does not fit yet), with the other waiting jobs of its structure key (up to
        ``group_max`` members, as many as fit), freeing idle pooled registers when that makes
        them fit."""
        queue = sorted(self.waiting)
        for w in queue:
            group = [w]
            key = w.prep.get("key")
            if key is not None:
                group += [o for o in queue if o is not w and o.prep.get("key") == key][: self.group_max - 1]
            while group:
                shape = group_shape(group, self.precision)
                need = sum(g.need for g in group)
                reg = self.pool.take(shape)
                extra = need - (register_bytes(*shape) if reg is not None else 0)
                if self.used + extra > self.budget and self.pool.bytes:
                    self.used -= self.pool.evict(self.used + extra - self.budget)
                if self.used + extra <= self.budget:
                    for g in group:
                        self.waiting.remove(g)
                    heapq.heapify(self.waiting)
                    self.used += extra
                    return group, reg
                if reg is not None:  # not admitted: the register goes back to the pool
                    self.pool.give(reg)
                group.pop()  # fewer members, then try again
        return None

    def _worker(self) -> None:
        _lib.ensure_device(self.device)
        while True:
            with self.cv:
                picked = None
                while not self.closed:
                    picked = self._admit() if self.waiting else None
                    if picked is not None:
                        break
                    self.cv.wait(0.05)
                if picked is None:
                    return
            group, reg = picked
            shape = group_shape(group, self.precision)
            need = sum(g.need for g in group)
            t_start = time.perf_counter()
            try:
                if reg is None:
                    reg = _lib.Register(*shape)
                results = execute_group([g.prep for g in group], self.precision, reg)
                t_end = time.perf_counter()
                for g, res in zip(group, results, strict=True):
                    res["latency_s"] = t_end - g.prep["t0"]
                    # where the latency went: host preparation (in the process pool, including its
                    # queue), waiting for a slot and memory, running (device work, host sampling)
                    res["prep_s"] = g.prep["t_prepared"] - g.prep["t0"]
                    res["wait_s"] = t_start - g.prep["t_prepared"]
                    res["run_s"] = t_end - t_start
                    g.future.set_result(res)
            except Exception as exc:  # noqa: BLE001 - handed to the client
                for g in group:
                    if not g.future.done():
                        g.future.set_exception(exc)
            finally:
                with self.cv:
                    if reg is not None:  # the register stays allocated, idle in the pool
                        self.pool.give(reg)
                        self.used -= need - register_bytes(*shape)
                    else:
                        self.used -= need
                    self.cv.notify_all()

    def close(self) -> None:
        """Stop the workers and free the device memory; jobs that have not run get a
        ``RuntimeError('server closed')``."""
        with self.cv:
            self.closed = True
            self.cv.notify_all()
        for t in self.threads:
            t.join(timeout=60)
        self.prep.shutdown(wait=True, cancel_futures=True)
        with self.cv:
            left, self.waiting = self.waiting, []
        for w in left:
            if not w.future.done():
                w.future.set_exception(RuntimeError("server closed"))
        with self.cv:
            self.used -= self.pool.clear()

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
    parts = {k: np.array([r.get(k, np.nan) for r in results]) for k in ("prep_s", "wait_s", "run_s", "apply_s", "reduce_s")}
    return {
        "results": results,
        "elapsed_s": elapsed,
        "circuits_per_s": len(jobs) / elapsed,
        "p50_s": float(np.percentile(lat, 50)),
        "p99_s": float(np.percentile(lat, 99)),
        "phases": {k: _phase_summary(v) for k, v in parts.items() if np.isfinite(v).any()},
    }


def _phase_summary(v: np.ndarray) -> dict[str, float]:
    """p50, p99 and mean of one phase's times over the jobs that report it."""
    v = v[np.isfinite(v)]
    return {"p50_s": float(np.percentile(v, 50)), "p99_s": float(np.percentile(v, 99)), "mean_s": float(v.mean())}
