"""Dynamic Clifford circuits on the device, one tableau per shot (``stabilizer.py:653-694``).

The noiseless gate prefix is simulated once; the rest of the circuit becomes a small program
(gates with Pauli noise, measurements with readout errors, resets, if/else with jump targets) that
one CTA runs shot after shot, drawing from the run's generator exactly as Orrery's shot loop does:
doubles for noise and readout, ``integers(2)`` (a buffered uint32) for random measurement outcomes.
"""

from __future__ import annotations

import ctypes as C
from typing import Any

import numpy as np

from lucivant_sim_gb300._lib import check, library
from lucivant_sim_gb300.stabilizer import CGATE, Encoder

SHOT_OP = np.dtype(
    [("code", "<i2"), ("noise", "<i2"), ("a", "<i2"), ("b", "<i2"), ("c", "<i2"), ("clbit", "<i2"),
     ("aux", "<i4"), ("nq", "<i2"), ("pad0", "<i2"), ("pad1", "<i4")]
)  # fmt: skip
SHOT_COND = np.dtype([("n", "<i4"), ("negate", "<i4"), ("value", "<u8"), ("bits", "<i4", (64,))])
assert SHOT_OP.itemsize == 24 and SHOT_COND.itemsize == 272

MEASURE, RESET, IF, ELSE, ENDIF = 100, 101, 102, 103, 104


def _sig(lib: C.CDLL) -> Any:
    fn = lib.lsg_per_shot_run
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_void_p, C.c_int64, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                   C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_int32, C.c_int64, C.c_void_p, C.c_void_p]  # fmt: skip
    return fn


def compile_program(circuit: Any, noise: Any) -> tuple[list[Any], Encoder, list[dict], list[tuple], list[tuple]]:
    ops = circuit.operations
    prefix: list[Any] = []
    start = 0
    for op in ops:
        if op.kind == "gate" and (noise is None or noise.gate_error(op.name, op.qubits) is None):
            prefix.append(op)
            start += 1
        elif op.kind in ("barrier", "gphase"):
            start += 1
        else:
            break
    enc = Encoder(noise)
    rows: list[dict] = []
    conds: list[tuple] = []
    readout: list[tuple] = []

    def emit(seq: Any) -> None:
        for op in seq:
            kind = op.kind
            if kind == "gate":
                code, k = enc.gate_code(op)
                qs = list(op.qubits) + [0, 0]
                rows.append(dict(code=code, noise=enc.noise_code(op), a=qs[0], b=qs[1], c=qs[2], nq=k, clbit=-1))
            elif kind == "measure":
                err = noise.readout_error(op.qubit) if noise else None
                r = -1
                if err is not None:
                    r = len(readout)
                    readout.append((err.p01, err.p10))
                rows.append(dict(code=MEASURE, a=op.qubit, clbit=-1 if op.clbit is None else op.clbit, noise=r))
            elif kind == "reset":
                rows.append(dict(code=RESET, a=op.qubit, clbit=-1, noise=-1))
            elif kind == "if":
                cond = op.condition
                conds.append((list(cond.clbits), int(cond.value), int(cond.negate)))
                at_if = len(rows)
                rows.append(dict(code=IF, c=len(conds) - 1, clbit=-1, noise=-1))
                emit(op.then)
                if op.otherwise:
                    at_else = len(rows)
                    rows.append(dict(code=ELSE, clbit=-1, noise=-1))
                    rows[at_if]["aux"] = len(rows)
                    emit(op.otherwise)
                    rows.append(dict(code=ENDIF, clbit=-1, noise=-1))
                    rows[at_else]["aux"] = len(rows) - 1
                else:
                    rows.append(dict(code=ENDIF, clbit=-1, noise=-1))
                    rows[at_if]["aux"] = len(rows) - 1
            # barrier, gphase: nothing on a tableau

    emit(ops[start:])
    return prefix, enc, rows, conds, readout


def per_shot(circuit: Any, shots: int, noise: Any, rng: np.random.Generator) -> dict[int, int]:
    """Counts keyed by the classical bits as an integer; leaves ``rng`` where Orrery's loop does."""
    if circuit.num_clbits > 256:
        from lucivant_sim_gb300._lib import SimulationError

        raise SimulationError("per-shot stabilizer runs keep at most 256 classical bits")
    lib = library()
    fn = _sig(lib)
    prefix_ops, enc, rows, conds, readout = compile_program(circuit, noise)
    prefix = enc.encode(prefix_ops, False) if prefix_ops else np.zeros(1, dtype=CGATE)
    prog = np.zeros(max(len(rows), 1), dtype=SHOT_OP)
    for i, row in enumerate(rows):
        for k, v in row.items():
            prog[i][k] = v
    cond_arr = np.zeros(max(len(conds), 1), dtype=SHOT_COND)
    for i, (bits, value, negate) in enumerate(conds):
        cond_arr[i]["n"] = len(bits)
        cond_arr[i]["value"] = value
        cond_arr[i]["negate"] = negate
        cond_arr[i]["bits"][: len(bits)] = bits
    ro = np.array(readout if readout else [(0.0, 0.0)], dtype=np.float64).reshape(-1)
    tables = enc.table_bytes()
    nt = enc.noise_array()
    st = rng.bit_generator.state
    s, inc = st["state"]["state"], st["state"]["inc"]
    m64 = (1 << 64) - 1
    state = np.array([s >> 64, s & m64, inc >> 64, inc & m64, st["has_uint32"], st["uinteger"], 0], dtype=np.uint64)
    out = np.zeros((shots, 4), dtype=np.uint64)
    check(fn(circuit.num_qubits, prefix.ctypes.data, len(prefix_ops), prog.ctypes.data, len(rows), tables.ctypes.data,
             len(enc.tables), nt.ctypes.data, len(enc.noise_rows), ro.ctypes.data, len(readout), cond_arr.ctypes.data,
             len(conds), circuit.num_clbits, shots, state.ctypes.data, out.ctypes.data))  # fmt: skip
    st["state"]["state"] = (int(state[0]) << 64) | int(state[1])
    st["has_uint32"] = int(state[4])
    st["uinteger"] = int(state[5])
    rng.bit_generator.state = st
    tally: dict[int, int] = {}
    for row in out:
        key = int(row[0]) | (int(row[1]) << 64) | (int(row[2]) << 128) | (int(row[3]) << 192)
        tally[key] = tally.get(key, 0) + 1
    return tally
