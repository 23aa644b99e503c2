"""Oracle (test infrastructure): the Clifford tables of Orrery's stabilizer engine, restated here
so the oracle does not lean on the product's host tables. Not shipped; never called by the product.

What it restates (``src/lucivant_sim/stabilizer.py``):

* ``conjugation_table``: how a k-qubit gate U conjugates each local Pauli P (``:52-118``). Index
  convention as the reference: a Pauli's bits (x0, z0, x1, z1, ...) read as a binary number, first
  qubit most significant, Y = (1, 1); the matrix is rounded to 12 decimals first and a gate is
  refused (None) when an image is not ±1 times one Pauli to 1e-8.
* ``kind_of``: the standard gates the reference gives named rules (``:122-147``).
* ``pauli_noise``: a mixture channel as cumulative branch probabilities and Pauli bits
  (``:150-184``), with the reference's arithmetic (cumulative sum, then divided by the total).
* ``clifford_problem``: the reference's walk over the gates in order (``:446-467``).

The derivation differs from the reference's (and from the product's): instead of projecting
U P U† onto all 4^k Paulis, it reads the image's Pauli directly off the matrix. A Pauli string
i^(x·z) X^x Z^z has one non-zero entry per column, at row c XOR x, of value i^(x·z) (-1)^(z·c);
so x is the row of column 0's non-zero entry, each z bit is the sign ratio of the column with
that bit set, and the whole image is then checked entrywise against the candidate.
"""

from __future__ import annotations

from dataclasses import dataclass
from functools import lru_cache
from typing import Any

import numpy as np
from numpy.typing import NDArray

MAX_QUBITS = 2048  # stabilizer.py:37
MAX_GATE_QUBITS = 3  # stabilizer.py:39
_TOL = 1e-8


@dataclass(frozen=True)
class Table:
    """``bits[i]`` = the image of Pauli i as (x0, z0, x1, z1, ...); ``sign[i]`` = 1 for a minus."""

    k: int
    bits: NDArray[np.uint8]
    sign: NDArray[np.uint8]


def _pauli_matrix(x: int, z: int, k: int) -> NDArray[np.complex128]:
    """i^(x·z) X^x Z^z on k qubits, x and z as k-bit integers (first qubit most significant)."""
    d = 1 << k
    cols = np.arange(d)
    m = np.zeros((d, d), dtype=np.complex128)
    signs = np.array([-1.0 if bin(z & c).count("1") & 1 else 1.0 for c in range(d)])
    m[cols ^ x, cols] = signs * (1j ** bin(x & z).count("1"))
    return m


def _label_bits(x: int, z: int, k: int) -> NDArray[np.uint8]:
    out = np.zeros(2 * k, dtype=np.uint8)
    for q in range(k):
        shift = k - 1 - q
        out[2 * q] = (x >> shift) & 1
        out[2 * q + 1] = (z >> shift) & 1
    return out


def _as_pauli(m: NDArray[np.complex128], k: int) -> tuple[int, int, complex] | None:
    """(x, z, c) with m = c · i^(x·z) X^x Z^z within 1e-8, or None."""
    d = 1 << k
    x = int(np.argmax(np.abs(m[:, 0])))
    lead = m[x, 0]
    if abs(lead) < 0.5:
        return None
    z = 0
    for q in range(k):
        col = 1 << (k - 1 - q)
        ratio = m[col ^ x, col] / lead
        if ratio.real < 0:
            z |= col
    c = lead / (1j ** bin(x & z).count("1"))
    if np.max(np.abs(m - c * _pauli_matrix(x, z, k))) > _TOL * d:
        return None
    return x, z, complex(c)


@lru_cache(maxsize=1024)
def _table_of(raw: bytes, k: int) -> Table | None:
    u = np.frombuffer(raw, dtype=np.complex128).reshape(1 << k, 1 << k)
    n = 1 << (2 * k)
    bits = np.zeros((n, 2 * k), dtype=np.uint8)
    sign = np.zeros(n, dtype=np.uint8)
    for i in range(n):
        px = pz = 0
        for q in range(k):  # label bits of Pauli i: qubit q's (x, z) at (2q, 2q + 1), MSB first
            shift = 2 * (k - 1 - q)
            px |= ((i >> (shift + 1)) & 1) << (k - 1 - q)
            pz |= ((i >> shift) & 1) << (k - 1 - q)
        image = u @ _pauli_matrix(px, pz, k) @ u.conj().T
        found = _as_pauli(image, k)
        if found is None:
            return None
        x, z, c = found
        if abs(abs(c) - 1) > _TOL or abs(c.imag) > _TOL:
            return None
        bits[i] = _label_bits(x, z, k)
        sign[i] = 1 if c.real < 0 else 0
    return Table(k, bits, sign)


def conjugation_table(matrix: NDArray[np.complex128]) -> Table | None:
    """The conjugation table of a gate matrix, or None when it is not Clifford (or too wide)
    (``stabilizer.py:83-118``)."""
    k = matrix.shape[0].bit_length() - 1
    if not 0 < k <= MAX_GATE_QUBITS:
        return None
    rounded = np.round(np.ascontiguousarray(matrix, dtype=np.complex128), 12) + 0.0
    return _table_of(rounded.tobytes(), k)


def _standard() -> dict[tuple[int, bytes, bytes], str]:
    h = np.array([[1, 1], [1, -1]]) / np.sqrt(2)
    named = {
        "h": h,
        "s": np.diag([1, 1j]),
        "sdg": np.diag([1, -1j]),
        "x": np.array([[0, 1], [1, 0]]),
        "y": np.array([[0, -1j], [1j, 0]]),
        "z": np.diag([1, -1]),
        "id": np.eye(2),
        "cx": np.eye(4)[[0, 1, 3, 2]],  # the first (most significant) qubit controls
        "cz": np.diag([1, 1, 1, -1]),
    }
    out = {}
    for name, m in named.items():
        t = conjugation_table(np.asarray(m, dtype=np.complex128))
        assert t is not None
        out[(t.k, t.bits.tobytes(), t.sign.tobytes())] = name
    return out


_KINDS = _standard()


def kind_of(table: Table) -> str | None:
    """The standard gate a table is (h, s, sdg, x, y, z, id, cx, cz), or None
    (``stabilizer.py:122-147``)."""
    return _KINDS.get((table.k, table.bits.tobytes(), table.sign.tobytes()))


def pauli_label(matrix: NDArray[np.complex128]) -> list[tuple[int, int]] | None:
    """(x, z) bits per qubit of a Pauli-string matrix up to a unit phase (first qubit first)
    (``stabilizer.py:150-158``)."""
    k = matrix.shape[0].bit_length() - 1
    found = _as_pauli(np.asarray(matrix, dtype=np.complex128), k)
    if found is None or abs(abs(found[2]) - 1) > _TOL:
        return None
    x, z, _c = found
    return [(int((x >> (k - 1 - q)) & 1), int((z >> (k - 1 - q)) & 1)) for q in range(k)]


@dataclass(frozen=True)
class PauliNoise:
    cumulative: NDArray[np.float64]
    branches: tuple[tuple[tuple[int, int], ...], ...]


def pauli_noise(channel: Any) -> PauliNoise | None:
    """Branches of a mixture channel whose operators are all Pauli strings, else None
    (``stabilizer.py:169-184``)."""
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


def gates(ops: Any) -> list[Any]:
    """Every gate of an operation list, if/else branches included, in order (``stabilizer.py:446-454``)."""
    out: list[Any] = []
    for op in ops:
        if op.kind == "gate":
            out.append(op)
        elif op.kind == "if":
            out += gates(op.then) + gates(op.otherwise)
    return out


def clifford_problem(circuit: Any, noise: Any = None) -> str | None:
    """Why the stabilizer engine cannot run ``circuit`` exactly, or None, one gate at a time
    (``stabilizer.py:457-467``)."""
    if circuit.num_qubits > MAX_QUBITS:
        return f"it has {circuit.num_qubits} qubits; the stabilizer engine allows up to {MAX_QUBITS}"
    seen: dict[int, bool] = {}
    for g in gates(circuit.operations):
        ok = seen.get(id(g.matrix))
        if ok is None:
            ok = seen[id(g.matrix)] = conjugation_table(g.matrix) is not None
        if not ok:
            return f"{g.name} on qubits {list(g.qubits)} isn't a Clifford gate"
        ch = noise.gate_error(g.name, g.qubits) if noise else None
        if ch is not None and pauli_noise(ch) is None:
            return f"the {ch.name} noise after {g.name} isn't a Pauli channel"
    return None
