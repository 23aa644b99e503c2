"""Host-side Clifford tables for the stabilizer engine.

A gate matrix is classified once into its Pauli-conjugation table (how U P U† maps each local
Pauli), and a noise channel into Pauli branches; these small tables are what the tableau and
frame kernels consume. The index convention — Pauli bits (x0, z0, x1, z1, ...) with the first
qubit most significant, Y as x = z = 1 — and the refusal messages follow
``src/lucivant_sim/stabilizer.py:48-187`` and ``:457-471``.
"""

from __future__ import annotations

import itertools
import operator
from dataclasses import dataclass
from functools import cached_property, lru_cache
from typing import Any

import numpy as np
from numpy.typing import NDArray

MAX_STABILIZER_QUBITS = 2048
MAX_CLIFFORD_GATE_QUBITS = 3

_ONE_QUBIT = {
    (0, 0): np.eye(2, dtype=np.complex128),
    (1, 0): np.array([[0, 1], [1, 0]], dtype=np.complex128),
    (1, 1): np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    (0, 1): np.array([[1, 0], [0, -1]], dtype=np.complex128),
}


@dataclass(frozen=True)
class CliffordMap:
    """``bits[i]`` is the image of Pauli i as (x0, z0, x1, z1, ...); ``sign[i]`` = 1 for a minus."""

    k: int
    bits: NDArray[np.uint8]
    sign: NDArray[np.uint8]


@lru_cache(maxsize=4)
def _basis(k: int) -> tuple[NDArray[np.uint8], NDArray[np.complex128]]:
    labels = np.array(list(itertools.product((0, 1), repeat=2 * k)), dtype=np.uint8)
    mats = []
    for row in labels:
        m = np.ones((1, 1), dtype=np.complex128)
        for q in range(k):
            m = np.kron(m, _ONE_QUBIT[(int(row[2 * q]), int(row[2 * q + 1]))])
        mats.append(m)
    return labels, np.stack(mats)


@lru_cache(maxsize=1024)
def _map_of(raw: bytes, k: int) -> CliffordMap | None:
    u = np.frombuffer(raw, dtype=np.complex128).reshape(1 << k, 1 << k)
    labels, mats = _basis(k)
    d = 1 << k
    bits = np.zeros((len(labels), 2 * k), dtype=np.uint8)
    sign = np.zeros(len(labels), dtype=np.uint8)
    for i, p in enumerate(mats):
        image = u @ p @ u.conj().T
        # overlap with every Pauli: tr(Q† image) / d
        overlaps = np.einsum("qji,ji->q", mats.conj(), image) / d
        j = int(np.argmax(np.abs(overlaps)))
        c = overlaps[j]
        if abs(abs(c) - 1) > 1e-8 or abs(c.imag) > 1e-8:
            return None
        bits[i] = labels[j]
        sign[i] = 1 if c.real < 0 else 0
    return CliffordMap(k, bits, sign)


_SEEN: dict[bytes, CliffordMap | None] = {}


def clifford_map(matrix: NDArray[np.complex128]) -> CliffordMap | None:
    """The conjugation table of a gate matrix, or None when it isn't Clifford (or too wide)."""
    key = np.ascontiguousarray(matrix).tobytes()
    if key in _SEEN:
        return _SEEN[key]
    k = matrix.shape[0].bit_length() - 1
    found = None
    if 0 < k <= MAX_CLIFFORD_GATE_QUBITS:
        rounded = np.round(np.ascontiguousarray(matrix, dtype=np.complex128), 12) + 0.0
        found = _map_of(rounded.tobytes(), k)
    if len(_SEEN) < 4096:
        _SEEN[key] = found
    return found


def _named_kinds() -> dict[tuple[int, bytes, bytes], str]:
    r = 1 / np.sqrt(2)
    named = {
        "h": np.array([[r, r], [r, -r]]),
        "s": np.diag([1, 1j]),
        "sdg": np.diag([1, -1j]),
        "x": np.array([[0, 1], [1, 0]]),
        "y": np.array([[0, -1j], [1j, 0]]),
        "z": np.diag([1, -1]),
        "id": np.eye(2),
        "cx": np.eye(4)[[0, 1, 3, 2]],
        "cz": np.diag([1, 1, 1, -1]),
    }
    table = {}
    for label, m in named.items():
        k = m.shape[0].bit_length() - 1
        cmap = _map_of((np.round(np.asarray(m, dtype=np.complex128), 12) + 0.0).tobytes(), k)
        assert cmap is not None
        table[(k, cmap.bits.tobytes(), cmap.sign.tobytes())] = label
    return table


_KINDS = _named_kinds()


def kind_of(cmap: CliffordMap) -> str | None:
    """The standard gate a table is (h, s, sdg, x, y, z, id, cx, cz), or None for the generic path."""
    return _KINDS.get((cmap.k, cmap.bits.tobytes(), cmap.sign.tobytes()))


def pauli_label(matrix: NDArray[np.complex128]) -> list[tuple[int, int]] | None:
    """(x, z) bits per qubit of a Pauli-string matrix (first qubit first), or None."""
    k = matrix.shape[0].bit_length() - 1
    labels, mats = _basis(k)
    overlaps = np.einsum("qji,ij->q", mats.conj(), matrix) / (1 << k)
    j = int(np.argmax(np.abs(overlaps)))
    if abs(abs(overlaps[j]) - 1) > 1e-8:
        return None
    return [(int(labels[j][2 * i]), int(labels[j][2 * i + 1])) for i in range(k)]


@dataclass(frozen=True)
class PauliNoise:
    """Branches of a Pauli channel: cumulative probabilities (normalised) and per-branch bits."""

    cumulative: NDArray[np.float64]
    branches: tuple[tuple[tuple[int, int], ...], ...]


@lru_cache(maxsize=256)
def pauli_noise(channel: Any) -> PauliNoise | None:
    if channel.mixture is None:
        return None
    probs, branches = [], []
    for p, m in channel.mixture:
        label = pauli_label(m)
        if label is None:
            return None
        probs.append(p)
        branches.append(tuple(label))
    return PauliNoise(np.cumsum(probs) / sum(probs), tuple(branches))


def all_gates(ops: Any) -> list[Any]:
    found: list[Any] = []
    for op in ops:
        if op.kind == "gate":
            found.append(op)
        elif op.kind == "if":
            found += all_gates(op.then)
            found += all_gates(op.otherwise)
    return found


class GateColumns:
    """Per-gate fields of a long gate list as columns, each read once on first use with C-level
    iteration (``map`` over ``attrgetter``): names, qubit tuples, arities, matrix identities
    (gates that share a matrix object share its analysis) and name indices. A columnar circuit
    gives them from its arrays instead (:meth:`from_arrays`): no gate object is read."""

    def __init__(self, gates: Any) -> None:
        self.gates = gates
        self.n = len(gates)

    @classmethod
    def from_arrays(cls, gates: Any, kind: np.ndarray, kind_names: list[str], qubits: np.ndarray,
                    arity: np.ndarray) -> GateColumns:  # fmt: skip
        """Columns of gates given as arrays: ``kind[i]`` indexes the distinct gates (one matrix
        object and one name each), ``qubits[i, :arity[i]]`` are gate i's qubits. ``gates`` is a
        sequence that builds gate i on access (only the first gate of each kind is read)."""
        self = cls(gates)
        kind = np.asarray(kind, dtype=np.int64)
        present = np.flatnonzero(np.bincount(kind, minlength=len(kind_names)))
        rank = np.zeros(len(kind_names), dtype=np.int64)
        rank[present] = np.arange(present.size)
        first = np.array([int(np.argmax(kind == k)) for k in present], dtype=np.int64)
        # names numbered in order of first appearance, as the per-gate reading numbers them
        by_appearance = [kind_names[int(present[j])] for j in np.argsort(first, kind="stable")]
        name_index = {name: i for i, name in enumerate(dict.fromkeys(by_appearance))}
        kind_name_id = np.array([name_index.get(name, -1) for name in kind_names], dtype=np.int64)
        self.__dict__.update(
            arity=np.asarray(arity, dtype=np.int64),
            matrix_ids=kind,
            matrix_groups=(first, rank[kind]),
            name_ids=kind_name_id[kind],
        )
        self._qmat = np.asarray(qubits, dtype=np.int64)
        self._kind_names = kind_names
        self._kind_name_id = kind_name_id
        return self

    @cached_property
    def names(self) -> list[str]:
        if hasattr(self, "_qmat"):
            return [self._kind_names[k] for k in self.matrix_ids.tolist()]
        return list(map(_NAME, self.gates))

    @cached_property
    def qubits(self) -> list[tuple[int, ...]]:
        if hasattr(self, "_qmat"):
            return [tuple(row[:a]) for row, a in zip(self._qmat.tolist(), self.arity.tolist(), strict=True)]
        return list(map(_QUBITS, self.gates))

    @cached_property
    def arity(self) -> np.ndarray:
        return np.fromiter(map(len, self.qubits), dtype=np.int64, count=self.n)

    @cached_property
    def matrix_ids(self) -> np.ndarray:
        return np.fromiter(map(id, map(_MATRIX, self.gates)), dtype=np.int64, count=self.n)

    @cached_property
    def matrix_groups(self) -> tuple[np.ndarray, np.ndarray]:
        """(index of each distinct matrix's first gate, per gate the index of its matrix)."""
        _u, first, inv = np.unique(self.matrix_ids, return_index=True, return_inverse=True)
        return first, inv

    @cached_property
    def name_arity_groups(self) -> tuple[np.ndarray, np.ndarray]:
        """Gates grouped by (name, arity), the key noise rules by gate name depend on: (index of
        each group's first gate, per gate its group), groups in ascending key order."""
        if hasattr(self, "_qmat"):  # from the distinct gates: key per kind, then per gate
            first_k, inv_k = self.matrix_groups
            kind_key = self._kind_name_id[self.matrix_ids[first_k]] * 64 + self.arity[first_k]
            uk, rank = np.unique(kind_key, return_inverse=True)
            first = np.array([int(first_k[rank == r].min()) for r in range(uk.size)], dtype=np.int64)
            return first, rank[inv_k]
        key = self.name_ids * 64 + self.arity
        _u, first, inv = np.unique(key, return_index=True, return_inverse=True)
        return first, inv

    @cached_property
    def name_ids(self) -> np.ndarray:
        name_id = {name: i for i, name in enumerate(dict.fromkeys(self.names))}
        return np.fromiter(map(name_id.__getitem__, self.names), dtype=np.int64, count=self.n)

    @cached_property
    def _flat(self) -> tuple[np.ndarray, np.ndarray]:
        flat = np.fromiter(itertools.chain.from_iterable(self.qubits), dtype=np.int64, count=int(self.arity.sum()))
        start = np.concatenate(([0], np.cumsum(self.arity)[:-1])).astype(np.int64)
        return flat, start

    def position(self, j: int) -> np.ndarray:
        """Qubit j of every gate as int16 (0 where a gate has fewer than j + 1 qubits)."""
        if hasattr(self, "_qmat"):
            if j >= self._qmat.shape[1]:
                return np.zeros(self.n, dtype=np.int16)
            return np.where(self.arity > j, self._qmat[:, j], 0).astype(np.int16)
        flat, start = self._flat
        has = self.arity > j
        at = np.where(has, start + j, 0)
        vals = flat[at] if flat.size else np.zeros_like(at)
        return np.where(has, vals, 0).astype(np.int16)


_NAME = operator.attrgetter("name")
_QUBITS = operator.attrgetter("qubits")
_MATRIX = operator.attrgetter("matrix")


def gates_and_columns(circuit: Any) -> tuple[list[Any], GateColumns]:
    """A circuit's gates and their columns: the circuit's own cached ones when it keeps them,
    else read here (circuits of other packages)."""
    cols = getattr(circuit, "gate_columns", None)
    if not isinstance(cols, GateColumns):
        cols = GateColumns(all_gates(circuit.operations))
    return cols.gates, cols


def first_index(keys: list[Any]) -> dict[Any, int]:
    """Each distinct key with the index of its first occurrence, in order of first occurrence."""
    n = len(keys)
    earliest = dict(zip(reversed(keys), range(n - 1, -1, -1)))  # the last write is the first index
    return dict(sorted(earliest.items(), key=lambda kv: kv[1]))


def clifford_problem(circuit: Any, noise: Any = None, gates: list[Any] | None = None,
                     cols: GateColumns | None = None) -> str | None:
    """Why the stabilizer engine can't run ``circuit`` exactly, or None."""
    if circuit.num_qubits > MAX_STABILIZER_QUBITS:
        return f"it has {circuit.num_qubits} qubits; the stabilizer engine allows up to {MAX_STABILIZER_QUBITS}"
    # circuits repeat their gate matrices and noise rules: check each distinct one once, at its
    # first gate; the problem reported is the one at the earliest gate (a gate's matrix before
    # its noise), as a walk over the gates in order would find it
    if gates is None:
        gates, cols = gates_and_columns(circuit)
    if not gates:
        return None
    cols = GateColumns(gates) if cols is None else cols
    firsts = cols.matrix_groups[0]
    bad_matrix = next((int(i) for i in np.sort(firsts) if clifford_map(gates[int(i)].matrix) is None), None)
    bad_noise, bad_channel = None, None
    if noise:
        by_arity = all(r.qubits is None for r in getattr(noise, "rules", []))
        if by_arity:
            candidates = [int(i) for i in np.sort(cols.name_arity_groups[0])]
        else:
            candidates = list(first_index(list(zip(cols.names, cols.qubits))).values())
        for i in candidates:
            if bad_matrix is not None and i > bad_matrix:
                break
            ch = noise.gate_error(gates[i].name, gates[i].qubits)
            if ch is not None and pauli_noise(ch) is None:
                bad_noise, bad_channel = i, ch
                break
    if bad_matrix is not None and (bad_noise is None or bad_matrix <= bad_noise):
        g = gates[bad_matrix]
        return f"{g.name} on qubits {list(g.qubits)} isn't a Clifford gate"
    if bad_noise is not None:
        return f"the {bad_channel.name} noise after {gates[bad_noise].name} isn't a Pauli channel"
    return None


def is_clifford(circuit: Any) -> bool:
    return clifford_problem(circuit) is None
