"""Trajectories (one statevector per shot) on the device.

The circuit and its noise become a flat device program (``lsg_traj_*`` in ``include/lsg.h``):
gates, mixture channels (branch picked from the shot's uniform, identity branches skipped as
``engines.py:168-169`` does), Kraus channels (Born-weighted pick, ``engines.py:172-183``),
measurements with readout flips (``simulator.py:300-306``), resets and if/else blocks.

Two modes:

* ``serial`` (the default, and what :func:`lucivant_sim_gb300.run` uses): shots run one after
  another on the device, all drawing from the run's NumPy generator in exactly Orrery's order
  (``simulator.py:364-371``), so counts are identical to Orrery's for the same seed (up to
  decisions whose uniform lies within 1e-12 of a device-computed threshold, which are counted).
* ``batched``: every shot is a member of one register and draws from its own row of uniforms
  (row b = the b-th block of ``max_draws`` uniforms of the run's generator). Seeded and
  reproducible, not Orrery's draw order; checked against the serial mode statistically.
"""

from __future__ import annotations

import ctypes as C
import os
from typing import Any

import numpy as np

from lucivant_sim_gb300 import _lib, engine
from lucivant_sim_gb300._lib import check, library, ptr

T_GATE, T_MIXTURE, T_KRAUS, T_MEASURE, T_RESET, T_SCALE, T_IF, T_ELSE, T_ENDIF = range(9)

TRAJ_DTYPE = np.dtype(
    [
        ("kind", "<i4"), ("opkind", "<i4"), ("nq", "<i4"), ("count", "<i4"), ("qubits", "<i4", (4,)),
        ("clbit", "<i4"), ("readout", "<i4"), ("negate", "<i4"), ("pad", "<i4"), ("data", "<i8"),
        ("value", "<u8"), ("p01", "<f8"), ("p10", "<f8"),
    ],
    align=True,
)  # fmt: skip
assert TRAJ_DTYPE.itemsize == 80

_SIGS = {
    "lsg_traj_create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.c_int64, C.c_int32,
                                  C.POINTER(C.c_void_p)]),
    "lsg_traj_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
    "lsg_traj_run_serial": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_double), C.c_int64,
                                      C.POINTER(C.c_uint64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "lsg_traj_run_batched": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_uint64),
                                       C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "lsg_traj_free": (C.c_int, [C.c_void_p]),
}  # fmt: skip

#: Uniforms staged per serial launch (the shots of one launch draw at most this many).
SERIAL_UNIFORMS = 1 << 24
#: Register bytes one batched launch may hold.
BATCH_BYTES = 16 << 30


def _lib_traj() -> C.CDLL:
    lib = library()
    if not getattr(lib, "_traj_sigs", False):
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype, fn.argtypes = res, args
        lib._traj_sigs = True
    return lib


class _Builder:
    def __init__(self) -> None:
        self.rows: list[dict[str, Any]] = []
        self.pool: list[np.ndarray] = []
        self.size = 0

    def data(self, arr: np.ndarray) -> int:
        flat = np.ascontiguousarray(arr, dtype=np.complex128).reshape(-1)
        at = self.size
        self.pool.append(flat)
        self.size += flat.size
        return at

    def add(self, **row: Any) -> None:
        self.rows.append(row)

    def packed(self) -> tuple[np.ndarray, np.ndarray]:
        table = np.zeros(len(self.rows), dtype=TRAJ_DTYPE)
        for i, row in enumerate(self.rows):
            for k, v in row.items():
                if k == "qubits":
                    table[i]["qubits"][: len(v)] = v
                else:
                    table[i][k] = v
            if "clbit" not in row:
                table[i]["clbit"] = -1
        pool = np.concatenate(self.pool) if self.pool else np.zeros(1, dtype=np.complex128)
        return table, np.ascontiguousarray(pool.view(np.float64))


def _mixture_data(channel: Any) -> tuple[int, np.ndarray]:
    """Running sums of the branch probabilities (the order ``engines.py:163-166`` adds them in),
    identity flags, then the branch matrices."""
    acc = 0.0
    cums, mats = [], []
    for p, u in channel.mixture:
        acc += p
        ident = bool(np.allclose(u, np.eye(u.shape[0])))
        cums.append(complex(acc, 1.0 if ident else 0.0))
        mats.append(np.asarray(u, dtype=np.complex128).reshape(-1))
    return len(cums), np.concatenate([np.array(cums, dtype=np.complex128), *mats])


def compile_ops(circuit: Any, noise: Any) -> tuple[np.ndarray, np.ndarray]:
    """The circuit's operation tree flattened into device trajectory operations."""
    b = _Builder()

    def walk(ops: Any) -> None:
        for op in ops:
            kind = op.kind
            if kind == "gate":
                opkind, data = engine.classify(op.matrix)
                qs = list(op.qubits)
                if len(qs) > 4:
                    raise engine.SimulationError(f"{op.name} acts on {len(qs)} qubits; trajectories take up to 4")
                b.add(kind=T_GATE, opkind=opkind, nq=len(qs), qubits=qs, data=b.data(data))
                ch = noise.gate_error(op.name, op.qubits) if noise else None
                if ch is None:
                    continue
                if len(qs) > 2:
                    raise engine.SimulationError(f"a {len(qs)}-qubit noise channel is wider than the trajectory engine's")
                if ch.mixture is not None:
                    count, data = _mixture_data(ch)
                    b.add(kind=T_MIXTURE, nq=len(qs), qubits=qs, count=count, data=b.data(data))
                else:
                    mats = np.concatenate([np.asarray(k, dtype=np.complex128).reshape(-1) for k in ch.kraus])
                    b.add(kind=T_KRAUS, nq=len(qs), qubits=qs, count=len(ch.kraus), data=b.data(mats))
            elif kind == "measure":
                err = noise.readout_error(op.qubit) if noise else None
                b.add(kind=T_MEASURE, nq=1, qubits=[op.qubit], clbit=-1 if op.clbit is None else op.clbit,
                      readout=int(err is not None), p01=err.p01 if err else 0.0, p10=err.p10 if err else 0.0)  # fmt: skip
            elif kind == "reset":
                b.add(kind=T_RESET, nq=1, qubits=[op.qubit])
            elif kind == "gphase":
                b.add(kind=T_SCALE, data=b.data(np.array([np.exp(1j * op.angle)])))
            elif kind == "if":
                cond = op.condition
                bits = np.array(list(cond.clbits), dtype=np.complex128)
                b.add(kind=T_IF, count=len(cond.clbits), value=int(cond.value), negate=int(cond.negate), data=b.data(bits))
                walk(op.then)
                if op.otherwise:
                    b.add(kind=T_ELSE)
                    walk(op.otherwise)
                b.add(kind=T_ENDIF)
            # barrier: nothing

    walk(circuit.operations)
    return b.packed()


class TrajectoryProgram:
    """A compiled trajectory program for registers of ``batch`` members."""

    def __init__(self, circuit: Any, noise: Any, precision: int, batch: int) -> None:
        self.lib = _lib_traj()
        self.n = circuit.num_qubits
        self.words = max(1, (circuit.num_clbits + 63) // 64)
        self.reg = engine.new_statevector(self.n, precision, batch)
        table, pool = compile_ops(circuit, noise)
        handle = C.c_void_p()
        check(self.lib.lsg_traj_create(self.reg.handle, table.ctypes.data, len(table), ptr(pool, C.c_double),
                                       pool.size // 2, circuit.num_clbits, C.byref(handle)))  # fmt: skip
        self.handle = handle
        md, steps = C.c_int64(0), C.c_int32(0)
        check(self.lib.lsg_traj_info(handle, C.byref(md), C.byref(steps)))
        self.max_draws, self.steps = int(md.value), int(steps.value)

    def run_serial(self, shots: int, uniforms: np.ndarray) -> tuple[np.ndarray, int, int]:
        out = np.zeros((max(shots, 1), self.words), dtype=np.uint64)
        consumed, near = C.c_int64(0), C.c_int64(0)
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        check(self.lib.lsg_traj_run_serial(self.handle, self.reg.handle, shots, ptr(u, C.c_double), u.size,
                                           ptr(out, C.c_uint64), C.byref(consumed), C.byref(near)))  # fmt: skip
        return out[:shots], int(consumed.value), int(near.value)

    def run_batched(self, uniforms: np.ndarray) -> tuple[np.ndarray, np.ndarray, int]:
        batch = self.reg.batch
        u = np.ascontiguousarray(uniforms, dtype=np.float64).reshape(batch, -1)
        out = np.zeros((batch, self.words), dtype=np.uint64)
        consumed = np.zeros(batch, dtype=np.int64)
        near = C.c_int64(0)
        check(self.lib.lsg_traj_run_batched(self.handle, self.reg.handle, ptr(u, C.c_double), u.shape[1],
                                            ptr(out, C.c_uint64), ptr(consumed, C.c_int64), C.byref(near)))  # fmt: skip
        return out, consumed, int(near.value)

    def free(self) -> None:
        if getattr(self, "handle", None):
            self.lib.lsg_traj_free(self.handle)
            self.handle = None
        self.reg.free()

    def __del__(self) -> None:
        try:
            self.free()
        except Exception:
            pass


def _key(words: np.ndarray) -> int:
    v = 0
    for i, w in enumerate(words):
        v |= int(w) << (64 * i)
    return v


def _tally(rows: np.ndarray, tally: dict[int, int]) -> None:
    if rows.shape[1] == 1:
        keys, counts = np.unique(rows[:, 0], return_counts=True)
        for k, c in zip(keys, counts, strict=True):
            tally[int(k)] = tally.get(int(k), 0) + int(c)
        return
    for r in rows:
        k = _key(r)
        tally[k] = tally.get(k, 0) + 1


def _generator_at(rng: np.random.Generator, position: int) -> np.random.Generator:
    """A copy of ``rng`` advanced by ``position`` doubles (one raw PCG64 draw each)."""
    bg = np.random.PCG64()
    bg.state = rng.bit_generator.state
    bg.advance(position)
    return np.random.Generator(bg)


def run_shots(circuit: Any, shots: int, noise: Any, rng: np.random.Generator, precision: int,
              mode: str | None = None) -> tuple[dict[int, int], dict[str, Any]]:  # fmt: skip
    """Counts keyed by the classical bits as an integer, and a report. Leaves ``rng`` where
    Orrery's shot loop leaves it (serial mode)."""
    mode = mode or os.environ.get("LSG_TRAJ_MODE", "serial")
    tally: dict[int, int] = {}
    report: dict[str, Any] = {"mode": mode, "near_threshold": 0}
    if shots == 0:
        return tally, report
    if mode == "serial":
        prog = TrajectoryProgram(circuit, noise, precision, 1)
        try:
            per = max(prog.max_draws, 1)
            chunk = max(1, min(shots, SERIAL_UNIFORMS // per))
            position = 0
            done = 0
            while done < shots:
                k = min(chunk, shots - done)
                u = _generator_at(rng, position).random(k * per)
                rows, consumed, near = prog.run_serial(k, u)
                _tally(rows, tally)
                position += consumed
                report["near_threshold"] += near
                done += k
            rng.bit_generator.advance(position)
            report["uniforms"] = position
        finally:
            prog.free()
        return tally, report
    if mode != "batched":
        raise ValueError("trajectory mode must be 'serial' or 'batched'")
    elt = 16 if precision == _lib.C128 else 8
    per_member = elt << circuit.num_qubits
    batch = int(max(1, min(shots, 65535, BATCH_BYTES // per_member)))
    prog = TrajectoryProgram(circuit, noise, precision, batch)
    try:
        per = max(prog.max_draws, 1)
        done = 0
        while done < shots:
            k = min(batch, shots - done)
            u = rng.random((batch, per))
            rows, _, near = prog.run_batched(u)
            _tally(rows[:k], tally)
            report["near_threshold"] += near
            done += k
    finally:
        prog.free()
    return tally, report
