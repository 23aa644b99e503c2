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
from lucivant_sim_gb300 import noise as nm_mod
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


_OFFDIAG: dict[int, np.ndarray] = {}
_CLASSIFIED: dict[bytes, tuple[int, np.ndarray]] = {}  # multi-qubit matrices (every cx shares one)


def classify(m: np.ndarray) -> tuple[int, np.ndarray]:
    """(kind, data) for a gate matrix: diagonal, phased permutation, or dense. The data of a
    multi-qubit matrix is shared between calls with equal matrices: callers only read it."""
    m = np.asarray(m, dtype=np.complex128)
    d = m.shape[0]
    if d == 2:  # the common one-qubit case without array passes
        a, b, c, e = m.ravel().tolist()
        if b == 0 and c == 0:
            return OP_DIAG, np.array([a, e])
        if a == 0 and e == 0 and b != 0 and c != 0:
            return OP_PERM, np.array([b, c, 1.0, 0.0], dtype=np.complex128)
        return OP_MATRIX, m
    key = m.tobytes()
    hit = _CLASSIFIED.get(key)
    if hit is None:
        hit = _classify_wide(m.copy(), d)
        hit[1].setflags(write=False)  # shared between callers
        if len(_CLASSIFIED) < 4096:
            _CLASSIFIED[key] = hit
    return hit


def _classify_wide(m: np.ndarray, d: int) -> tuple[int, np.ndarray]:
    nz = m != 0
    off = _OFFDIAG.get(d)
    if off is None:
        off = _OFFDIAG[d] = ~np.eye(d, dtype=bool)
    if not np.any(nz & off):
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

    gate_errors = nm_mod.GateErrors(noises)
    errors_of: dict[tuple[str, tuple[int, ...]], list[Any]] = {}
    for op in circuit.operations:
        if op.kind == "gate":
            qs = tuple(op.qubits)
            u = np.asarray(op.matrix, dtype=np.complex128)
            chans = errors_of.get((op.name, qs))
            if chans is None:
                chans = errors_of[(op.name, qs)] = gate_errors(op.name, qs)
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


# ---------------------------------------------------------------------------- Pauli-transfer form
#
# A density register in Pauli-transfer form holds r_P = Tr(P rho) for every n-qubit Pauli P: real,
# 4^n of them, in a register of 2n bits where qubit q's Pauli digit sits in bits (n+q, q) = (x, z)
# (I = 00, Z = 01, X = 10, Y = 11). A channel E on k qubits acts as the real 4^k x 4^k matrix
# R[P', P] = 2^-k Tr(P' E(P)) on the digits of its qubits, listed (x bits, then z bits) the way
# the vectorised form lists (row bits, then column bits). Half the bytes of the complex
# vectorised form, and a one-qubit channel costs 4 real multiply-adds per element instead of 16.

PAULI_DIGITS = (
    np.eye(2, dtype=np.complex128),  # I: x=0 z=0
    np.array([[1, 0], [0, -1]], dtype=np.complex128),  # Z: x=0 z=1
    np.array([[0, 1], [1, 0]], dtype=np.complex128),  # X: x=1 z=0
    np.array([[0, -1j], [1j, 0]], dtype=np.complex128),  # Y: x=1 z=1
)

REAL_OF = {_lib.C128: _lib.R64, _lib.C64: _lib.R32}


def _pauli_basis(k: int) -> list[np.ndarray]:
    """The 4^k Paulis in digit-index order: index bits (x_0..x_{k-1}, z_0..z_{k-1}), MSB first;
    qubit 0 of the operator is the most significant tensor factor (as in gate matrices)."""
    out = []
    for j in range(4**k):
        xs = [(j >> (2 * k - 1 - i)) & 1 for i in range(k)]
        zs = [(j >> (k - 1 - i)) & 1 for i in range(k)]
        m = np.ones((1, 1), dtype=np.complex128)
        for x, z in zip(xs, zs, strict=True):
            m = np.kron(m, PAULI_DIGITS[2 * x + z])
        out.append(m)
    return out


_BASIS_CACHE: dict[int, np.ndarray] = {}


def _paulis(k: int) -> np.ndarray:
    """The 4^k Paulis stacked, shape (4^k, 2^k, 2^k) (cached)."""
    hit = _BASIS_CACHE.get(k)
    if hit is None:
        hit = _BASIS_CACHE[k] = np.stack(_pauli_basis(k))
    return hit


_BASIS_T_CACHE: dict[int, np.ndarray] = {}


def _paulis_t(k: int) -> np.ndarray:
    """vec(P_a^T) for the 4^k Paulis, shape (4^k, 4^k) (cached)."""
    hit = _BASIS_T_CACHE.get(k)
    if hit is None:
        p = _paulis(k)
        hit = _BASIS_T_CACHE[k] = np.ascontiguousarray(p.transpose(0, 2, 1).reshape(len(p), -1))
    return hit


def ptm_of_kraus_stack(kraus: np.ndarray) -> np.ndarray:
    """Real Pauli-transfer matrices of channels given as Kraus stacks, shape (..., nk, d, d):
    R[a, c] = d^-1 sum_K Tr(P_a K P_c K^dagger), as (..., d^2, d^2)."""
    d = kraus.shape[-1]
    k = d.bit_length() - 1
    p = _paulis(k)
    n4 = len(p)
    # E(P_c) = sum_n K_n P_c K_n^dagger for every c, then R[a, c] = d^-1 vec(P_a^T) . vec(E(P_c))
    kk = kraus[..., :, None, :, :]
    e = (kk @ p @ np.swapaxes(kk, -1, -2).conj()).sum(axis=-4)
    bt = _paulis_t(k)
    r = (bt @ np.swapaxes(e.reshape(*e.shape[:-2], d * d), -1, -2)) / d
    if r.shape[-2:] != (n4, n4):
        raise AssertionError("Pauli-transfer shape")
    if np.max(np.abs(r.imag), initial=0.0) > 1e-12:
        raise SimulationError("a channel without a real Pauli-transfer matrix (not Hermiticity-preserving)")
    return np.ascontiguousarray(r.real)


def ptm_of_superop(s: np.ndarray, k: int) -> np.ndarray:
    """Real Pauli-transfer matrix of a superoperator given on vectorised (row-major) matrices."""
    p = _paulis(k)
    b = p.reshape(len(p), -1)
    # R[a, c] = 2^-k Tr(P_a E(P_c)) = 2^-k sum_ij P_a[j, i] E(P_c)[i, j] = 2^-k vec(P_a^T) . (S vec(P_c))
    bt = p.transpose(0, 2, 1).reshape(len(p), -1)
    r = (bt @ s @ b.T) / (1 << k)
    if np.max(np.abs(r.imag), initial=0.0) > 1e-12:
        raise SimulationError("a channel without a real Pauli-transfer matrix (not Hermiticity-preserving)")
    return np.ascontiguousarray(r.real)


def ptm_of_unitary(u: np.ndarray) -> np.ndarray:
    return ptm_of_kraus_stack(np.asarray(u, dtype=np.complex128)[None])


def ptm_of_kraus(kraus: Any, k: int) -> np.ndarray:
    return ptm_of_kraus_stack(np.stack([np.asarray(m, dtype=np.complex128) for m in kraus]))


def ptm_depolarizing(p: float, k: int) -> np.ndarray:
    """(1-p) rho + p I/d Tr rho: r_I kept, every other coefficient scaled by 1-p."""
    d = np.full(4**k, 1.0 - p)
    d[0] = 1.0
    return np.diag(d)


def _renames(src: np.ndarray, nbits: int) -> list[tuple[str, int, int]] | None:
    """Decompose a permutation of bit patterns (out[r] = in[src[r]]) that is linear over GF(2)
    into bit CX / SWAP renames, in application order: [("cx", control, target) | ("swap", a, b)]
    on operator positions (0 = most significant). None when src is not linear."""
    d = 1 << nbits
    if src[0] != 0:
        return None
    for r in range(d):
        acc = 0
        for pbit in range(nbits):
            if (r >> pbit) & 1:
                acc ^= int(src[1 << pbit])
        if acc != int(src[r]):
            return None

    def vec(x: int) -> list[int]:
        return [(x >> (nbits - 1 - p)) & 1 for p in range(nbits)]

    # B[:, p] = vec(src(e_p)) where e_p has only position p set
    cols = [vec(int(src[1 << (nbits - 1 - p)])) for p in range(nbits)]
    b = np.array(cols, dtype=np.uint8).T  # b[row, col]
    steps: list[tuple[str, int, int]] = []  # column operations F_1.. reducing B to I
    for i in range(nbits):
        piv = next(j for j in range(i, nbits) if b[i, j])
        if piv != i:
            b[:, [i, piv]] = b[:, [piv, i]]
            steps.append(("swap", i, piv))
        for c in range(nbits):
            if c != i and b[i, c]:
                b[:, c] ^= b[:, i]
                steps.append(("cx", c, i))  # F = I + E[i, c]: adds column i into column c
    assert (b == np.eye(nbits, dtype=np.uint8)).all()
    return steps[::-1]


_CX_SRC = np.array([1, 1, 1, 1, 0, 1, 3, 2], dtype=np.complex128)  # unit phases, src [0, 1, 3, 2]
_SWAP_SRC = np.array([1, 1, 1, 1, 0, 2, 1, 3], dtype=np.complex128)


def _snap(x: np.ndarray) -> np.ndarray:
    """Rounding residue of the transfer-matrix products (|x| ~ 1e-16) snapped to the exact 0 and
    +-1 entries it stands for, so trace preservation and permutation structure are recognised."""
    x = np.asarray(x, dtype=np.float64)
    r = np.rint(x)  # the candidate: |x| < 1e-14 -> 0, ||x| - 1| < 1e-14 -> sign(x)
    keep = (np.abs(x - r) >= 1e-14) | (np.abs(r) > 1.0)
    return np.where(keep, x, r + 0.0)  # + 0.0: -0.0 becomes 0.0


def ptm_capable(circuit: Any, noises: list[Any]) -> bool:
    """The Pauli-transfer form takes gates and channels on up to two qubits (wider ones would be
    4^k-dense real operators); otherwise the complex vectorised form is used."""
    for op in circuit.operations:
        if op.kind == "gate" and len(op.qubits) > 2:
            return False
    return True


def _ptm_entries(mats: np.ndarray) -> list[tuple[str, Any]]:
    """Classify a stack of Pauli-transfer operators, ``mats`` (gates, members, d, d), each as the
    cheapest kind that represents it exactly: ("diag", diagonals), ("perm", (bit renames,
    phases)) — a GF(2)-linear permutation of digit patterns with signs — or ("dense", matrices),
    each with a leading member axis. Structure is read with rounding residue taken as zero and
    only the data kept is snapped (:func:`_snap`)."""
    g, _m, d, _ = mats.shape
    idx = np.arange(d)
    a = np.abs(mats)
    big, small = a.max(axis=1) >= 1e-14, a.min(axis=1) >= 1e-14  # (gates, d, d)
    nz_all = big  # the union of the members' patterns
    same = (small | ~big).all(axis=(1, 2))  # every member has the union's pattern
    diag_only = ~(nz_all & ~np.eye(d, dtype=bool)).any(axis=(1, 2))
    perm_like = (nz_all.sum(axis=2) == 1).all(axis=1) & (nz_all.sum(axis=1) == 1).all(axis=1) & same
    out: list[tuple[str, Any] | None] = [None] * g
    dense = []
    for i in range(g):
        if diag_only[i]:
            out[i] = ("diag", _snap(mats[i][:, idx, idx]))
            continue
        if perm_like[i]:
            src = nz_all[i].argmax(axis=1)
            steps = _renames(src, d.bit_length() - 1)
            if steps is not None:
                out[i] = ("perm", (steps, _snap(mats[i][:, idx, src])))
                continue
        dense.append(i)
    if dense:
        snapped = _snap(mats[dense])
        for j, i in enumerate(dense):
            out[i] = ("dense", snapped[j])
    return out  # type: ignore[return-value]


def _emit_ptm(ops: OpList, bits: list[int], entry: tuple[str, Any]) -> None:
    """Append one classified Pauli-transfer operator: shared by all members when their data
    agree, per member otherwise; identity diagonals are left out."""
    kind, val = entry
    if kind == "diag":
        if (val == val[0]).all():
            if not np.all(val[0] == 1.0):
                ops.add(OP_DIAG, bits, val[0].astype(np.complex128))
        else:
            ops.add_batched(OP_DIAG, bits, val.astype(np.complex128))
    elif kind == "perm":
        steps, phases = val
        for k, a, b in steps:
            ops.add(OP_PERM, [bits[a], bits[b]], _CX_SRC if k == "cx" else _SWAP_SRC)
        if (phases == phases[0]).all():
            if not np.all(phases[0] == 1.0):
                ops.add(OP_DIAG, bits, phases[0].astype(np.complex128))
        else:
            ops.add_batched(OP_DIAG, bits, phases.astype(np.complex128))
    elif (val == val[0]).all():
        ops.add(OP_MATRIX, bits, val[0].astype(np.complex128))
    else:
        ops.add_batched(OP_MATRIX, bits, val.astype(np.complex128))


def ptm_oplist(circuit: Any, noises: list[Any]) -> OpList:
    """The noisy static evolution of :func:`dm_oplist` as Pauli-transfer operators: each gate
    with its channel is ONE real operator on the (x, z) digits of its qubits. Channel matrices are
    formed once per distinct channel; the gates' transfer matrices, their products with the
    channels and the classification run over all gates sharing a channel stack at once."""
    n = circuit.num_qubits
    cache: dict[tuple[int, ...], np.ndarray] = {}

    def chan_stack(chans: list[Any], k: int, key: tuple[int, ...]) -> np.ndarray:
        hit = cache.get(key)  # keyed by the channels' ids: the noise models hold them for this call
        if hit is None:
            mats = np.empty((len(chans), 4**k, 4**k))
            todo: dict[int, list[int]] = {}
            for i, ch in enumerate(chans):
                if ch.analytic_depolarizing:
                    mats[i] = ptm_depolarizing(ch.params[0], k)
                else:
                    todo.setdefault(len(ch.kraus), []).append(i)
            for _nk, members in todo.items():  # one product per Kraus count
                kr = np.array([chans[i].kraus for i in members], dtype=np.complex128)
                mats[members] = ptm_of_kraus_stack(kr)
            hit = cache[key] = mats
        return hit

    # 1. the gates and resets in order, grouped by (arity, channel stack)
    gate_errors = nm_mod.GateErrors(noises)
    chans_of: dict[tuple[str, tuple[int, ...]], tuple[list[Any], tuple[int, ...]]] = {}  # channels per gate signature
    items: list[tuple[list[int], tuple[Any, ...], int]] = []  # (bits, group key, index in group)
    groups: dict[tuple[Any, ...], list[np.ndarray]] = {}
    uniq: dict[tuple[Any, ...], dict[bytes, int]] = {}
    for op in circuit.operations:
        if op.kind == "gate":
            qs = tuple(op.qubits)
            k = len(qs)
            if k > 2:
                raise SimulationError("the Pauli-transfer form takes gates on up to two qubits")
            sig = (op.name, qs)
            got = chans_of.get(sig)
            if got is None:
                chans = gate_errors(op.name, qs)
                got = chans_of[sig] = (chans, tuple(id(ch) for ch in chans))
            chans, chan_key = got
            present = [c is not None for c in chans]
            if any(present) and not all(present):
                raise ValueError("batched noise models must attach channels to the same gates")
            gkey = ("gate", k, chan_key if chans[0] is not None else None)
            if gkey not in groups:
                groups[gkey] = []
                if chans[0] is not None:
                    chan_stack(chans, k, chan_key)
            u = np.asarray(op.matrix, dtype=np.complex128)
            ukey = u.tobytes()  # equal gates (every cx) share their product and classification
            at = uniq.setdefault(gkey, {}).get(ukey)
            if at is None:
                at = uniq[gkey][ukey] = len(groups[gkey])
                groups[gkey].append(u)
            items.append(([n + q for q in qs] + list(qs), gkey, at))
        elif op.kind == "reset":
            items.append(([n + op.qubit, op.qubit], ("reset",), 0))
            groups.setdefault(("reset",), [])
        # measurements are deferred; a global phase leaves a density matrix unchanged
    # 2. per group: the gates' transfer matrices in one product, composed with the channel stack
    entries: dict[tuple[Any, ...], list[tuple[str, Any]]] = {}
    for gkey, us in groups.items():
        if gkey[0] == "reset":
            entries[gkey] = _ptm_entries(ptm_of_kraus(RESET_KRAUS, 1)[None, None])
            continue
        r_gates = ptm_of_kraus_stack(np.stack(us)[:, None])  # (gates, d, d)
        if gkey[2] is None:
            mats = r_gates[:, None]
        else:
            mats = cache[gkey[2]][None] @ r_gates[:, None]  # (gates, members, d, d)
        entries[gkey] = _ptm_entries(mats)
    # 3. the operators in circuit order
    ops = OpList()
    for bits, gkey, i in items:
        _emit_ptm(ops, bits, entries[gkey][i])
    return ops


def ptm_to_density_ops(n: int) -> OpList:
    """Per-qubit change of basis from Pauli-transfer coefficients (loaded as real amplitudes of a
    complex register) to the vectorised density matrix: rho[row, col] = 2^-n sum_P r_P P[row, col]."""
    t = np.zeros((4, 4), dtype=np.complex128)
    for d, pm in enumerate(PAULI_DIGITS):
        for row in range(2):
            for col in range(2):
                t[2 * row + col, d] = pm[row, col] / 2
    ops = OpList()
    for q in range(n):
        ops.add(OP_MATRIX, [n + q, q], t)
    return ops


def dm_form(circuit: Any, noises: list[Any]) -> str:
    """"ptm" (the default) or "superop", from ``LSG_DM_FORM`` and what the circuit needs."""
    want = os.environ.get("LSG_DM_FORM", "ptm")
    if want not in ("ptm", "superop"):
        raise ValueError("LSG_DM_FORM must be ptm or superop")
    return "ptm" if want == "ptm" and ptm_capable(circuit, noises) else "superop"


def evolve_density(circuit: Any, noises: list[Any], precision: int) -> _lib.Register:
    """A density register (one member per noise model) evolved through ``circuit``."""
    n = circuit.num_qubits
    if dm_form(circuit, noises) == "ptm":
        reg = new_density(n, REAL_OF[precision], len(noises))
        reg.apply_from_basis(ptm_oplist(circuit, noises))
    else:
        reg = new_density(n, precision, len(noises))
        reg.apply_from_basis(dm_oplist(circuit, noises))
    return reg


def density_download(reg: _lib.Register, member: int = 0) -> np.ndarray:
    """Member ``member`` of a density register as a (2^n, 2^n) complex128 matrix."""
    n = reg.nbits // 2
    if reg.precision in (_lib.C128, _lib.C64):
        return reg.download()[member].reshape(1 << n, 1 << n)
    with _lib.Register(reg.nbits, _lib.C128) as out:
        reg.to_complex(member, out)
        out.apply(ptm_to_density_ops(n))
        return out.download()[0].reshape(1 << n, 1 << n)


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
    """A density register of n qubits: complex vectorised (C128/C64) or Pauli-transfer (R64/R32)."""
    if n > MAX_DENSITY_QUBITS:
        raise SimulationError(
            f"{n} qubits need more memory than the density-matrix engine allows "
            f"(up to {MAX_DENSITY_QUBITS}); use method='trajectories'"
        )
    return _lib.Register(2 * n, precision, batch)
