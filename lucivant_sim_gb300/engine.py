"""Circuits and noise to device operator lists, and the device-side exact answers.

A statevector circuit becomes one ``lsg_apply`` call (the library fuses it into tile passes).
A noisy circuit on the density matrix becomes superoperators on the 2n-bit register:

* a one-qubit gate with its channel is ONE 4x4 operator on bits (n+q, q):
  S = Σ_k K⊗K̄ · (U⊗Ū), formed in FP64 (the analytic depolarising form of
  ``engines.py:122-135`` written as its 4x4 superoperator);
* a wider gate is U on its row bits and Ū on its column bits (``engines.py:233-235``), followed by
  the channel: the analytic depolarising operator for depolarising channels (``engines.py:242-244``)
  or the superoperator Σ_k K⊗K̄ of any other Kraus channel (``engines.py:245-250``);
* a reset is the two-Kraus channel of ``engines.py:252-255``.

Matrices are classified the way ``_apply_slices`` does (``engines.py:58-60``): diagonal, a
permutation with phases (moves only), or general.
"""

from __future__ import annotations

import os
from typing import Any

import numpy as np

from lucivant_sim_gb300 import _lib
from lucivant_sim_gb300._lib import OP_DEPOL, OP_DIAG, OP_MATRIX, OP_PERM, OP_SCALE, OpList, SimulationError

MAX_STATEVECTOR_QUBITS = 26
MAX_DENSITY_QUBITS = 13
RESET_KRAUS = (
    np.array([[1, 0], [0, 0]], dtype=np.complex128),
    np.array([[0, 1], [0, 0]], dtype=np.complex128),
)

PRECISIONS = {"c128": _lib.C128, "complex128": _lib.C128, "c64": _lib.C64, "complex64": _lib.C64}


def precision_code(precision: str | None) -> int:
    """Precision by name; the default comes from ``LSG_PRECISION`` (else complex128)."""
    name = precision or os.environ.get("LSG_PRECISION", "c128")
    try:
        return PRECISIONS[name]
    except KeyError:
        raise ValueError(f"precision must be one of {', '.join(PRECISIONS)}") from None


def classify(m: np.ndarray) -> tuple[int, np.ndarray]:
    """(kind, data) for a gate matrix: diagonal, phased permutation, or dense."""
    m = np.asarray(m, dtype=np.complex128)
    nz = m != 0
    d = m.shape[0]
    if not np.any(nz & ~np.eye(d, dtype=bool)):
        return OP_DIAG, np.diagonal(m).copy()
    if bool((nz.sum(axis=1) == 1).all() and (nz.sum(axis=0) == 1).all()):
        src = nz.argmax(axis=1)
        phases = m[np.arange(d), src]
        return OP_PERM, np.concatenate([phases, src.astype(np.complex128)])
    return OP_MATRIX, m


def superop(kraus: Any) -> np.ndarray:
    """Σ_k K ⊗ K̄: the channel on the (row bits, column bits) of a vectorised density matrix."""
    total = None
    for k in kraus:
        k = np.asarray(k, dtype=np.complex128)
        term = np.kron(k, k.conj())
        total = term if total is None else total + term
    return total


def depolarizing_superop(p: float, k: int) -> np.ndarray:
    """(1-p) ρ + (p/d) I ⊗ Tr ρ as a matrix on (row bits, column bits), k = 1."""
    d = 1 << k
    s = (1 - p) * np.eye(d * d, dtype=np.complex128)
    diag = [(r << k) | r for r in range(d)]
    for a in diag:
        for b in diag:
            s[a, b] += p / d
    return s


def fuse_runs(ops: Any) -> list[Any]:
    """Consecutive one-qubit gates on a qubit merged into one (``simulator.py:196-226``);
    only for ideal statevector evolution."""
    out: list[Any] = []
    open_at: dict[int, int] = {}
    for op in ops:
        kind = op.kind
        if kind == "gate" and len(op.qubits) == 1:
            q = op.qubits[0]
            at = open_at.get(q)
            if at is not None:
                prev = out[at]
                out[at] = _Fused(q, np.asarray(op.matrix, dtype=np.complex128) @ np.asarray(prev.matrix, dtype=np.complex128))
                continue
            open_at[q] = len(out)
            out.append(op)
            continue
        if kind == "gate":
            for q in op.qubits:
                open_at.pop(q, None)
        elif kind in ("measure", "reset"):
            open_at.pop(op.qubit, None)
        elif kind in ("if", "barrier"):
            open_at.clear()
        out.append(op)
    return out


class _Fused:
    kind = "gate"
    name = "fused"

    def __init__(self, q: int, matrix: np.ndarray) -> None:
        self.qubits = (q,)
        self.matrix = matrix


def sv_oplist(circuit: Any, fuse: bool = True) -> OpList:
    """The static statevector evolution of ``_evolve`` (``simulator.py:229-251``) as operators."""
    ops = OpList()
    seq = fuse_runs(circuit.operations) if fuse else circuit.operations
    for op in seq:
        if op.kind == "gate":
            kind, data = classify(op.matrix)
            ops.add(kind, list(op.qubits), data)
        elif op.kind == "gphase":
            ops.add(OP_SCALE, [], np.array([np.exp(1j * op.angle)]))
    return ops


def _channel_ops(n: int, qubits: tuple[int, ...], channels: list[Any], ops: OpList) -> None:
    """Append the channel after a multi-qubit gate; one channel per batch member."""
    first = channels[0]
    k = len(qubits)
    bits = [n + q for q in qubits] + list(qubits)
    if first.analytic_depolarizing and k in (1, 2):
        vals = np.array([[ch.params[0]] for ch in channels], dtype=np.complex128)
        if len(channels) == 1:
            ops.add(OP_DEPOL, bits, vals[0])
        else:
            ops.add_batched(OP_DEPOL, bits, vals)
        return
    if 2 * k > 5:
        raise SimulationError(f"a {k}-qubit Kraus channel is wider than the density-matrix engine's operators")
    mats = np.stack([superop(ch.kraus) for ch in channels])
    if len(channels) == 1:
        ops.add(OP_MATRIX, bits, mats[0])
    else:
        ops.add_batched(OP_MATRIX, bits, mats)


def dm_oplist(circuit: Any, noises: list[Any]) -> OpList:
    """Noisy static evolution (``simulator.py:229-251`` with ``engines.py:233-255``) for one or more
    noise models (one per batch member, all with the same rule structure)."""
    n = circuit.num_qubits
    ops = OpList()
    batched = len(noises) > 1
    chan_cache: dict[int, tuple[Any, np.ndarray]] = {}

    def chan_superop(ch: Any) -> np.ndarray:
        hit = chan_cache.get(id(ch))
        if hit is None or hit[0] is not ch:
            s = depolarizing_superop(ch.params[0], 1) if ch.analytic_depolarizing else superop(ch.kraus)
            hit = chan_cache[id(ch)] = (ch, s)
        return hit[1]

    for op in circuit.operations:
        if op.kind == "gate":
            qs = tuple(op.qubits)
            u = np.asarray(op.matrix, dtype=np.complex128)
            chans = [nm.gate_error(op.name, qs) if nm is not None else None for nm in noises]
            present = [c is not None for c in chans]
            if any(present) and not all(present):
                raise ValueError("batched noise models must attach channels to the same gates")
            if len(qs) == 1:
                q = qs[0]
                gate_s = np.kron(u, u.conj())
                if chans[0] is None:
                    kind, data = classify(gate_s)
                    ops.add(kind, [n + q, q], data)
                    continue
                mats = [chan_superop(ch) @ gate_s for ch in chans]
                if batched:
                    ops.add_batched(OP_MATRIX, [n + q, q], np.stack(mats))
                else:
                    ops.add(OP_MATRIX, [n + q, q], mats[0])
                continue
            kind, data = classify(u)
            ops.add(kind, [n + q for q in qs], data)
            kind, data = classify(u.conj())
            ops.add(kind, list(qs), data)
            if chans[0] is not None:
                _channel_ops(n, qs, chans, ops)
        elif op.kind == "reset":
            ops.add(OP_MATRIX, [n + op.qubit, op.qubit], superop(RESET_KRAUS))
        # measurements are deferred; a global phase leaves a density matrix unchanged
    return ops


def pauli_masks(label: str) -> tuple[int, int]:
    """(x mask, z mask) of a Pauli label, qubit 0 rightmost; Y sets both."""
    xm = zm = 0
    for q, letter in enumerate(reversed(label.upper())):
        if letter in "XY":
            xm |= 1 << q
        if letter in "ZY":
            zm |= 1 << q
    return xm, zm


def new_statevector(n: int, precision: int = _lib.C128, batch: int = 1) -> _lib.Register:
    if n > MAX_STATEVECTOR_QUBITS:
        raise SimulationError(
            f"{n} qubits need more memory than the statevector engine allows (up to {MAX_STATEVECTOR_QUBITS})"
        )
    return _lib.Register(n, precision, batch)


def new_density(n: int, precision: int = _lib.C128, batch: int = 1) -> _lib.Register:
    if n > MAX_DENSITY_QUBITS:
        raise SimulationError(
            f"{n} qubits need more memory than the density-matrix engine allows "
            f"(up to {MAX_DENSITY_QUBITS}); use method='trajectories'"
        )
    return _lib.Register(2 * n, precision, batch)
