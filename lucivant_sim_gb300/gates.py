"""Gate matrices for the host side of the engine.

Conventions follow Orrery (``src/lucivant_sim/gates.py:1-7``): a k-qubit matrix has its first
qubit argument as the most significant bit, and results are little-endian (qubit 0 is the
rightmost bit of a bitstring). The table of names, parameter counts and arities mirrors
``src/lucivant_sim/gates.py:108-168`` so programs read the same; the matrices are written out here
from their textbook definitions.
"""

from __future__ import annotations

import cmath
import math
from collections.abc import Callable
from typing import NamedTuple

import numpy as np
from numpy.typing import NDArray

Matrix = NDArray[np.complex128]


def _c(rows: list[list[complex]]) -> Matrix:
    return np.array(rows, dtype=np.complex128)


I2 = np.eye(2, dtype=np.complex128)
X = _c([[0, 1], [1, 0]])
Y = _c([[0, -1j], [1j, 0]])
Z = _c([[1, 0], [0, -1]])
H = _c([[1, 1], [1, -1]]) / math.sqrt(2)
PAULIS: dict[str, Matrix] = {"I": I2, "X": X, "Y": Y, "Z": Z}


def rx(theta: float) -> Matrix:
    c, s = math.cos(theta / 2), math.sin(theta / 2)
    return _c([[c, -1j * s], [-1j * s, c]])


def ry(theta: float) -> Matrix:
    c, s = math.cos(theta / 2), math.sin(theta / 2)
    return _c([[c, -s], [s, c]])


def rz(theta: float) -> Matrix:
    return _c([[cmath.exp(-0.5j * theta), 0], [0, cmath.exp(0.5j * theta)]])


def phase(theta: float) -> Matrix:
    return _c([[1, 0], [0, cmath.exp(1j * theta)]])


def u3(theta: float, phi: float, lam: float) -> Matrix:
    c, s = math.cos(theta / 2), math.sin(theta / 2)
    return _c([[c, -cmath.exp(1j * lam) * s], [cmath.exp(1j * phi) * s, cmath.exp(1j * (phi + lam)) * c]])


def controlled(u: Matrix, controls: int = 1) -> Matrix:
    """``u`` acting when all ``controls`` leading (most significant) qubits are 1."""
    d = u.shape[0]
    full = d << controls
    out = np.eye(full, dtype=np.complex128)
    out[full - d :, full - d :] = u
    return out


def negcontrolled(u: Matrix) -> Matrix:
    """``u`` acting when the leading qubit is 0."""
    d = u.shape[0]
    out = np.eye(2 * d, dtype=np.complex128)
    out[:d, :d] = u
    return out


def pauli_string_matrix(labels: str) -> Matrix:
    out = np.ones((1, 1), dtype=np.complex128)
    for letter in labels:
        out = np.kron(out, PAULIS[letter])
    return out.astype(np.complex128)


def pauli_rotation(labels: str, theta: float) -> Matrix:
    """exp(-i theta/2 P) for a Pauli string P (first letter on the first qubit)."""
    p = pauli_string_matrix(labels)
    return math.cos(theta / 2) * np.eye(p.shape[0], dtype=np.complex128) - 1j * math.sin(theta / 2) * p


SX = _c([[1 + 1j, 1 - 1j], [1 - 1j, 1 + 1j]]) / 2
SWAP = _c([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]])
ISWAP = _c([[1, 0, 0, 0], [0, 0, 1j, 0], [0, 1j, 0, 0], [0, 0, 0, 1]])
ECR = ((np.kron(X, I2) - np.kron(Y, X)) / math.sqrt(2)).astype(np.complex128)
DCX = _c([[1, 0, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1], [0, 1, 0, 0]])


class GateSpec(NamedTuple):
    """A built-in gate: parameter count, qubit count, and a matrix builder."""

    params: int
    qubits: int
    build: Callable[..., Matrix]


def _const(m: Matrix) -> Callable[..., Matrix]:
    return lambda: m


_CX = controlled(X)
_CP = lambda t: controlled(phase(t))  # noqa: E731
_CCX = controlled(X, 2)
_CSWAP = controlled(SWAP)

GATES: dict[str, GateSpec] = {
    "id": GateSpec(0, 1, _const(I2)),
    "i": GateSpec(0, 1, _const(I2)),
    "x": GateSpec(0, 1, _const(X)),
    "y": GateSpec(0, 1, _const(Y)),
    "z": GateSpec(0, 1, _const(Z)),
    "h": GateSpec(0, 1, _const(H)),
    "s": GateSpec(0, 1, _const(phase(math.pi / 2))),
    "sdg": GateSpec(0, 1, _const(phase(-math.pi / 2))),
    "t": GateSpec(0, 1, _const(phase(math.pi / 4))),
    "tdg": GateSpec(0, 1, _const(phase(-math.pi / 4))),
    "sx": GateSpec(0, 1, _const(SX)),
    "sxdg": GateSpec(0, 1, _const(SX.conj().T)),
    "rx": GateSpec(1, 1, rx),
    "ry": GateSpec(1, 1, ry),
    "rz": GateSpec(1, 1, rz),
    "p": GateSpec(1, 1, phase),
    "phase": GateSpec(1, 1, phase),
    "u1": GateSpec(1, 1, phase),
    "u2": GateSpec(2, 1, lambda phi, lam: u3(math.pi / 2, phi, lam)),
    "u3": GateSpec(3, 1, u3),
    "u": GateSpec(3, 1, u3),
    "U": GateSpec(3, 1, u3),
    "cx": GateSpec(0, 2, _const(_CX)),
    "CX": GateSpec(0, 2, _const(_CX)),
    "cnot": GateSpec(0, 2, _const(_CX)),
    "cy": GateSpec(0, 2, _const(controlled(Y))),
    "cz": GateSpec(0, 2, _const(controlled(Z))),
    "ch": GateSpec(0, 2, _const(controlled(H))),
    "csx": GateSpec(0, 2, _const(controlled(SX))),
    "cp": GateSpec(1, 2, _CP),
    "cphase": GateSpec(1, 2, _CP),
    "cu1": GateSpec(1, 2, _CP),
    "crx": GateSpec(1, 2, lambda t: controlled(rx(t))),
    "cry": GateSpec(1, 2, lambda t: controlled(ry(t))),
    "crz": GateSpec(1, 2, lambda t: controlled(rz(t))),
    "cu3": GateSpec(3, 2, lambda a, b, c: controlled(u3(a, b, c))),
    "cu": GateSpec(4, 2, lambda a, b, c, g: controlled(cmath.exp(1j * g) * u3(a, b, c))),
    "swap": GateSpec(0, 2, _const(SWAP)),
    "iswap": GateSpec(0, 2, _const(ISWAP)),
    "ecr": GateSpec(0, 2, _const(ECR)),
    "dcx": GateSpec(0, 2, _const(DCX)),
    "rxx": GateSpec(1, 2, lambda t: pauli_rotation("XX", t)),
    "ryy": GateSpec(1, 2, lambda t: pauli_rotation("YY", t)),
    "rzz": GateSpec(1, 2, lambda t: pauli_rotation("ZZ", t)),
    "rzx": GateSpec(1, 2, lambda t: pauli_rotation("ZX", t)),
    "ccx": GateSpec(0, 3, _const(_CCX)),
    "toffoli": GateSpec(0, 3, _const(_CCX)),
    "ccz": GateSpec(0, 3, _const(controlled(Z, 2))),
    "cswap": GateSpec(0, 3, _const(_CSWAP)),
    "fredkin": GateSpec(0, 3, _const(_CSWAP)),
    "c3x": GateSpec(0, 4, _const(controlled(X, 3))),
    "c3sqrtx": GateSpec(0, 4, _const(controlled(SX, 3))),
    "c4x": GateSpec(0, 5, _const(controlled(X, 4))),
    "u0": GateSpec(1, 1, lambda _g: I2),
}

#: Other spellings and the canonical name that noise rules use (``gates.py:171-184``).
ALIASES: dict[str, str] = {
    "U": "u",
    "u3": "u",
    "CX": "cx",
    "cnot": "cx",
    "phase": "p",
    "u1": "p",
    "cphase": "cp",
    "cu1": "cp",
    "toffoli": "ccx",
    "fredkin": "cswap",
    "i": "id",
}


def canonical_name(name: str) -> str:
    return ALIASES.get(name, name)


def gate_matrix(name: str, params: tuple[float, ...]) -> Matrix:
    return GATES[name].build(*params)


def matrix_power(u: Matrix, k: float) -> Matrix:
    """u**k: whole powers by repeated products, fractional ones by eigen-decomposition."""
    if float(k).is_integer():
        n = int(k)
        return np.linalg.matrix_power(u if n >= 0 else u.conj().T, abs(n))
    vals, vecs = np.linalg.eig(u)
    return (vecs @ np.diag(vals**k) @ np.linalg.inv(vecs)).astype(np.complex128)
