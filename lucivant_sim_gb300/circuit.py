"""The circuit the engine runs: a flat list of operations with matrices already resolved.

Field names and ``kind`` tags match Orrery's IR (``src/lucivant_sim/circuit.py:21-81``), so the
engine also accepts circuits built by Orrery itself: everything below dispatches on ``op.kind``.
:meth:`Circuit.digest` hashes the same canonical JSON as ``circuit.py:165-199`` (matrices rounded
to 12 decimals), so a fingerprint names the same circuit in both projects.
"""

from __future__ import annotations

import hashlib
import json
from dataclasses import dataclass, field
from functools import cached_property
from typing import Any, Literal

import numpy as np

from lucivant_sim_gb300.gates import Matrix


@dataclass(frozen=True, eq=False)
class Gate:
    """A unitary on ``qubits``; the first qubit is the matrix's most significant bit."""

    name: str
    qubits: tuple[int, ...]
    matrix: Matrix
    params: tuple[float, ...] = ()
    kind: Literal["gate"] = "gate"


@dataclass(frozen=True)
class Measure:
    qubit: int
    clbit: int | None  # None: the outcome is discarded
    kind: Literal["measure"] = "measure"


@dataclass(frozen=True)
class Reset:
    qubit: int
    kind: Literal["reset"] = "reset"


@dataclass(frozen=True)
class Barrier:
    qubits: tuple[int, ...]
    kind: Literal["barrier"] = "barrier"


@dataclass(frozen=True)
class GlobalPhase:
    angle: float
    kind: Literal["gphase"] = "gphase"


@dataclass(frozen=True)
class Condition:
    """Holds when classical bits ``clbits`` (least significant first) read ``value``."""

    clbits: tuple[int, ...]
    value: int
    negate: bool = False

    def holds(self, bits: list[int]) -> bool:
        reading = 0
        for i, c in enumerate(self.clbits):
            reading |= bits[c] << i
        return (reading == self.value) != self.negate


@dataclass(frozen=True)
class IfElse:
    condition: Condition
    then: tuple[Any, ...]
    otherwise: tuple[Any, ...] = ()
    kind: Literal["if"] = "if"


Operation = Gate | Measure | Reset | Barrier | GlobalPhase | IfElse


@dataclass(frozen=True)
class Register:
    name: str
    offset: int
    size: int


_JSON_CACHE: dict[bytes, tuple[list[list[list[float]]], str]] = {}


def _matrix_json(matrix: np.ndarray) -> tuple[list[list[list[float]]], str]:
    """A matrix's canonical entries (rounded to 12 decimals, [re, im] pairs) and their compact
    JSON text, cached by the matrix's bytes (every cx of a circuit shares one entry)."""
    key = np.ascontiguousarray(matrix).tobytes()
    hit = _JSON_CACHE.get(key)
    if hit is None:
        rounded = np.round(np.asarray(matrix, dtype=np.complex128), 12) + 0.0  # folds -0.0 into 0.0
        entries = [[[float(v.real), float(v.imag)] for v in row] for row in rounded]
        hit = (entries, json.dumps(entries, separators=(",", ":")))
        if len(_JSON_CACHE) < 8192:
            _JSON_CACHE[key] = hit
    return hit


def _matrix_entries(matrix: np.ndarray) -> list[list[list[float]]]:
    return _matrix_json(matrix)[0]


def _op_record(op: Any) -> object:
    kind = op.kind
    if kind == "gate":
        return ["g", list(op.qubits), _matrix_entries(op.matrix)]
    if kind == "measure":
        return ["m", op.qubit, op.clbit]
    if kind == "reset":
        return ["r", op.qubit]
    if kind == "barrier":
        return ["b"]
    if kind == "gphase":
        return ["p", round(op.angle, 12)]
    cond = op.condition
    return [
        "if",
        [list(cond.clbits), cond.value, cond.negate],
        [_op_record(o) for o in op.then],
        [_op_record(o) for o in op.otherwise],
    ]


def is_dynamic(circuit: Any) -> bool:
    """True when outcomes feed conditions, or a qubit is used after being measured or reset
    mid-circuit (``circuit.py:121-138``): such circuits run one shot at a time."""
    ops = circuit.operations
    kinds = [op.kind for op in ops]
    # fast path: gates (and barriers, phases) first, then only measurements: static
    first = next((i for i, k in enumerate(kinds) if k not in ("gate", "barrier", "gphase")), len(kinds))
    if all(k in ("measure", "barrier") for k in kinds[first:]):
        return False
    touched: set[int] = set()
    finished: set[int] = set()
    for op in ops:
        kind = op.kind
        if kind == "if":
            return True
        if kind == "gate":
            if finished.intersection(op.qubits):
                return True
            touched.update(op.qubits)
        elif kind == "reset":
            if op.qubit in touched or op.qubit in finished:
                return True
        elif kind == "measure":
            finished.add(op.qubit)
    return False


def final_measurements(circuit: Any) -> list[tuple[int, int]]:
    """(qubit, clbit) pairs in program order of each clbit's first write; a later write to a
    clbit replaces the qubit (``circuit.py:140-146``)."""
    last: dict[int, int] = {}
    for op in circuit.operations:
        if op.kind == "measure" and op.clbit is not None:
            last[op.clbit] = op.qubit
    return [(q, c) for c, q in last.items()]


def format_bits(circuit: Any, bits: int) -> str:
    """Registers last-declared first, space separated, bit 0 of each on the right
    (``circuit.py:202-211``)."""
    if not circuit.cregs:
        return format(bits, f"0{circuit.num_clbits}b") if circuit.num_clbits else ""
    return " ".join(
        format((bits >> reg.offset) & ((1 << reg.size) - 1), f"0{reg.size}b") for reg in reversed(circuit.cregs)
    )


def format_bits_bytes(circuit: Any, values: np.ndarray) -> np.ndarray:
    """:func:`format_bits` of many packed outcomes (int64, fewer than 63 classical bits) as one
    fixed-width byte-string array (``S<width>``; ``S1`` of empty strings when there are no
    characters): the characters of every string are laid out in one byte array."""
    values = np.asarray(values, dtype=np.int64).reshape(-1)
    regs = list(reversed(circuit.cregs)) if circuit.cregs else [None]
    cols: list[np.ndarray] = []
    for i, reg in enumerate(regs):
        offset, size = (0, circuit.num_clbits) if reg is None else (reg.offset, reg.size)
        if i:
            cols.append(np.full((values.size, 1), ord(" "), dtype=np.uint8))
        if size:
            shifts = np.arange(offset + size - 1, offset - 1, -1, dtype=np.int64)  # most significant first
            cols.append((((values[:, None] >> shifts) & 1) + ord("0")).astype(np.uint8))
    width = sum(c.shape[1] for c in cols)
    if width == 0:
        return np.zeros(values.size, dtype="S1")
    chars = np.ascontiguousarray(np.concatenate(cols, axis=1))
    return chars.view(f"S{width}").ravel()


def format_bits_many(circuit: Any, values: np.ndarray) -> list[str]:
    """:func:`format_bits` of many packed outcomes (int64, fewer than 63 classical bits) at once."""
    return [b.decode() for b in format_bits_bytes(circuit, values)]


@dataclass(frozen=True)
class Circuit:
    num_qubits: int
    num_clbits: int
    operations: tuple[Any, ...]
    qregs: tuple[Register, ...] = ()
    cregs: tuple[Register, ...] = ()
    inputs: dict[str, float] = field(default_factory=dict)

    # Both scan every operation; the operations never change, so each is computed once per
    # circuit (a 2048-qubit Clifford workload holds four million of them).
    @cached_property
    def _dynamic(self) -> bool:
        return is_dynamic(self)

    @cached_property
    def _final(self) -> tuple[tuple[int, int], ...]:
        return tuple(final_measurements(self))

    @cached_property
    def gate_columns(self) -> Any:
        """Every gate (branches included) and its fields as columns
        (:class:`lucivant_sim_gb300.clifford.GateColumns`), read once per circuit and shared by the
        Clifford check and the stabilizer encoder."""
        from lucivant_sim_gb300.clifford import GateColumns, all_gates

        return GateColumns(all_gates(self.operations))

    def is_dynamic(self) -> bool:
        return self._dynamic

    def final_measurements(self) -> list[tuple[int, int]]:
        return list(self._final)

    def count_ops(self) -> dict[str, int]:
        tally: dict[str, int] = {}

        def walk(ops: tuple[Any, ...]) -> None:
            for op in ops:
                if op.kind == "if":
                    walk(op.then)
                    walk(op.otherwise)
                    continue
                key = op.name if op.kind == "gate" else op.kind
                tally[key] = tally.get(key, 0) + 1

        walk(self.operations)
        return dict(sorted(tally.items()))

    def canonical(self) -> dict[str, object]:
        return {
            "qubits": self.num_qubits,
            "clbits": self.num_clbits,
            "cregs": [[r.name, r.offset, r.size] for r in self.cregs],
            "ops": [_op_record(o) for o in self.operations],
        }

    def canonical_text(self) -> str:
        """``json.dumps(self.canonical(), separators=(",", ":"), sort_keys=True)``, assembled from
        cached per-matrix texts: the records are lists (only the top level is a dict, written in
        sorted key order), so joining the parts' compact texts gives the same characters."""
        parts = []
        for op in self.operations:
            if op.kind == "gate":
                qubits = ",".join(str(int(q)) for q in op.qubits)
                parts.append(f'["g",[{qubits}],{_matrix_json(op.matrix)[1]}]')
            else:
                parts.append(json.dumps(_op_record(op), separators=(",", ":"), sort_keys=True))
        cregs = json.dumps([[r.name, r.offset, r.size] for r in self.cregs], separators=(",", ":"))
        return (
            f'{{"clbits":{json.dumps(self.num_clbits)},"cregs":{cregs},"ops":[{",".join(parts)}],'
            f'"qubits":{json.dumps(self.num_qubits)}}}'
        )

    def digest(self) -> str:
        return "sha256:" + hashlib.sha256(self.canonical_text().encode()).hexdigest()

    def format_bits(self, bits: int) -> str:
        return format_bits(self, bits)


class ColumnarCircuit:
    """A static circuit held as arrays: gates, then measurements into classical bits.

    Gate i is distinct gate ``kind[i]`` (a name, a matrix object shared by all its gates, its
    parameters) on qubits ``qubits[i, :arity[i]]``. Built programmatically (a million-gate Clifford
    workload), it gives the stabilizer engine its gate columns straight from the arrays, so no
    per-gate object is made for a run; ``operations`` (and everything derived from it: digests,
    op counts) materialises the ordinary operation list on first use, the same as a
    :class:`Circuit` of those operations."""

    def __init__(self, num_qubits: int, num_clbits: int, kind_names: list[str], kind_matrices: list[Any],
                 kind: np.ndarray, qubits: np.ndarray, arity: np.ndarray, measures: list[tuple[int, int]],
                 qregs: tuple[Register, ...] = (), cregs: tuple[Register, ...] = (),
                 kind_params: list[tuple[float, ...]] | None = None) -> None:  # fmt: skip
        self.num_qubits, self.num_clbits = num_qubits, num_clbits
        self.kind_names, self.kind_matrices = list(kind_names), list(kind_matrices)
        self.kind_params = list(kind_params) if kind_params is not None else [()] * len(self.kind_names)
        self.kind = np.asarray(kind, dtype=np.int64)
        self.qubits = np.asarray(qubits, dtype=np.int64)
        self.arity = np.asarray(arity, dtype=np.int64)
        self.measures = [(int(q), int(c)) for q, c in measures]
        self.qregs, self.cregs = qregs, cregs
        self.inputs: dict[str, float] = {}

    def gate(self, i: int) -> Gate:
        k, a = int(self.kind[i]), int(self.arity[i])
        return Gate(self.kind_names[k], tuple(int(q) for q in self.qubits[i, :a]), self.kind_matrices[k],
                    self.kind_params[k])  # fmt: skip

    @cached_property
    def operations(self) -> tuple[Any, ...]:
        gates = [self.gate(i) for i in range(len(self.kind))]
        return tuple(gates) + tuple(Measure(q, c) for q, c in self.measures)

    @cached_property
    def _plain(self) -> Circuit:
        return Circuit(self.num_qubits, self.num_clbits, self.operations, self.qregs, self.cregs, {})

    @cached_property
    def gate_columns(self) -> Any:
        from lucivant_sim_gb300.clifford import GateColumns

        return GateColumns.from_arrays(_GateSequence(self), self.kind, self.kind_names, self.qubits, self.arity)

    def is_dynamic(self) -> bool:
        return False  # gates, then measurements only

    def final_measurements(self) -> list[tuple[int, int]]:
        last: dict[int, int] = {}
        for q, c in self.measures:
            last[c] = q
        return [(q, c) for c, q in last.items()]

    def count_ops(self) -> dict[str, int]:
        return self._plain.count_ops()

    def canonical(self) -> dict[str, object]:
        return self._plain.canonical()

    def canonical_text(self) -> str:
        return self._plain.canonical_text()

    def digest(self) -> str:
        return self._plain.digest()

    def format_bits(self, bits: int) -> str:
        return format_bits(self, bits)


class _GateSequence:
    """The gates of a columnar circuit as a read-only sequence, each built on access."""

    def __init__(self, circuit: ColumnarCircuit) -> None:
        self.circuit = circuit

    def __len__(self) -> int:
        return len(self.circuit.kind)

    def __getitem__(self, i: Any) -> Any:
        if isinstance(i, slice):
            return [self.circuit.gate(j) for j in range(*i.indices(len(self)))]
        if i < 0:
            i += len(self)
        if not 0 <= i < len(self):
            raise IndexError(i)
        return self.circuit.gate(i)

    def __iter__(self) -> Any:
        return (self.circuit.gate(i) for i in range(len(self)))
