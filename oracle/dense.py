"""Oracle (test infrastructure): NumPy restatement of Orrery's statevector, density-matrix,
sampling and trajectory paths. Not shipped; never called by the product.

States are flat little-endian arrays: bit q of the index is qubit q (``engines.py:8-9``). A
density matrix on n qubits is the flat 2n-bit vector of the row-major (d, d) matrix, so qubit q
is column bit q and row bit n+q (``engines.py:222-231``).
"""

from __future__ import annotations

import secrets
from typing import Any

import numpy as np
from numpy.typing import NDArray

C128 = NDArray[np.complex128]
X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
MAX_STATEVECTOR_QUBITS = 26
MAX_DENSITY_QUBITS = 13
AUTO_DENSITY_QUBITS = 10
AUTO_STABILIZER_QUBITS = 12
MAX_SHOTS = 10_000_000


class OracleError(RuntimeError):
    pass


# ------------------------------------------------------------------ gate application


def apply_bits(vec: C128, nbits: int, matrix: C128, bits: tuple[int, ...] | list[int]) -> C128:
    """A k-bit matrix on index bits ``bits`` (bits[0] = matrix MSB), out of place.

    Follows ``engines.py:38-42`` (the contraction) and, for one-bit general matrices, the
    batched (outer, 2, inner) product of ``engines.py:63-71``.
    """
    k = len(bits)
    if nbits == 0 or k == 0:
        return vec.copy()
    m = np.asarray(matrix, dtype=np.complex128)
    if k == 1:
        inner = 1 << bits[0]
        return np.matmul(m, vec.reshape(-1, 2, inner)).reshape(-1)
    t = vec.reshape([2] * nbits)
    axes = [nbits - 1 - b for b in bits]
    out = np.tensordot(m.reshape([2] * (2 * k)), t, axes=(list(range(k, 2 * k)), axes))
    return np.ascontiguousarray(np.moveaxis(out, list(range(k)), axes)).reshape(-1)


def depolarizing_trace(vec: C128, nbits: int, p: float, rows: list[int], cols: list[int]) -> C128:
    """(1-p) rho + (p/d) I ⊗ Tr_targets(rho) on the flat DM (``engines.py:122-135``)."""
    k = len(rows)
    d = 1 << k
    t = vec.reshape([2] * nbits)
    axes = [nbits - 1 - b for b in rows + cols]
    moved = np.moveaxis(t, axes, range(2 * k))
    mat = moved.reshape((d, d, *moved.shape[2 * k :]))
    partial = np.trace(mat, axis1=0, axis2=1)
    res = mat * (1 - p)
    for i in range(d):
        res[i, i] += (p / d) * partial
    return np.ascontiguousarray(np.moveaxis(res.reshape(moved.shape), range(2 * k), axes)).reshape(-1)


# -------------------------------------------------------------------- statevector


def sv_zero(n: int) -> C128:
    if n > MAX_STATEVECTOR_QUBITS:
        raise OracleError(f"{n} qubits need more memory than the statevector engine allows")
    v = np.zeros(1 << n, dtype=np.complex128)
    v[0] = 1
    return v


def fuse_runs(ops: tuple[Any, ...]) -> list[Any]:
    """Merge consecutive one-qubit gates per qubit (``simulator.py:196-226``)."""
    from types import SimpleNamespace

    out: list[Any] = []
    open_at: dict[int, int] = {}
    for op in ops:
        if op.kind == "gate" and len(op.qubits) == 1:
            (q,) = op.qubits
            at = open_at.get(q)
            if at is not None:
                prev = out[at]
                out[at] = SimpleNamespace(kind="gate", name="fused", qubits=(q,), matrix=op.matrix @ prev.matrix)
                continue
            open_at[q] = len(out)
            out.append(op)
            continue
        if op.kind == "gate":
            for q in op.qubits:
                open_at.pop(q, None)
        elif op.kind in ("measure", "reset"):
            open_at.pop(op.qubit, None)
        elif op.kind in ("if", "barrier"):
            open_at.clear()
        out.append(op)
    return out


def evolve_sv(circuit: Any) -> C128:
    """Static ideal evolution (``simulator.py:229-251``); measurements deferred."""
    n = circuit.num_qubits
    v = sv_zero(n)
    for op in fuse_runs(circuit.operations):
        if op.kind == "gate":
            v = apply_bits(v, n, op.matrix, [q for q in op.qubits])
        elif op.kind == "gphase":
            v = v * np.exp(1j * op.angle)
    return v


def evolve_dm(circuit: Any, noise: Any) -> C128:
    """Static noisy evolution of the flat DM (``simulator.py:229-251``, ``engines.py:233-255``)."""
    n = circuit.num_qubits
    if n > MAX_DENSITY_QUBITS:
        raise OracleError(f"{n} qubits need more memory than the density-matrix engine allows")
    nb = 2 * n
    rho = np.zeros(1 << nb, dtype=np.complex128)
    rho[0] = 1
    for op in circuit.operations:
        if op.kind == "gate":
            rows = [n + q for q in op.qubits]
            cols = list(op.qubits)
            rho = apply_bits(rho, nb, op.matrix, rows)
            rho = apply_bits(rho, nb, op.matrix.conj(), cols)
            ch = noise.gate_error(op.name, op.qubits) if noise else None
            if ch is not None:
                rho = dm_channel(rho, n, ch, op.qubits)
        elif op.kind == "reset":
            k0 = np.array([[1, 0], [0, 0]], dtype=np.complex128)
            k1 = np.array([[0, 1], [0, 0]], dtype=np.complex128)
            rho = dm_kraus(rho, n, (k0, k1), (op.qubit,))
    return rho


def dm_kraus(rho: C128, n: int, kraus: Any, qubits: tuple[int, ...]) -> C128:
    rows = [n + q for q in qubits]
    cols = list(qubits)
    total = None
    for k in kraus:
        term = apply_bits(apply_bits(rho, 2 * n, k, rows), 2 * n, k.conj(), cols)
        total = term if total is None else total + term
    return rho if total is None else total


def dm_channel(rho: C128, n: int, ch: Any, qubits: tuple[int, ...]) -> C128:
    if ch.analytic_depolarizing and len(qubits) in (1, 2):
        return depolarizing_trace(rho, 2 * n, ch.params[0], [n + q for q in qubits], list(qubits))
    return dm_kraus(rho, n, ch.kraus, qubits)


def dm_probabilities(rho: C128, n: int) -> NDArray[np.float64]:
    d = 1 << n
    return np.clip(rho.reshape(d, d).diagonal().real, 0.0, None).astype(np.float64)


def marginal(probs: NDArray[np.float64], n: int, qubits: list[int]) -> NDArray[np.float64]:
    """``engines.py:267-275``: index bit i is the i-th smallest of ``qubits``."""
    keep = sorted(qubits)
    if n == 0:
        return probs
    drop = tuple(n - 1 - q for q in range(n) if q not in keep)
    t = probs.reshape([2] * n)
    return np.asarray(t.sum(axis=drop) if drop else t).reshape(-1)


# ------------------------------------------------------------------------ sampling


def sample(circuit: Any, probs: NDArray[np.float64], shots: int, noise: Any, rng: np.random.Generator) -> dict[str, int]:
    """CDF search then readout flips then counting (``simulator.py:254-284``)."""
    pairs = circuit.final_measurements()
    if not pairs or shots == 0:
        return {}
    measured = sorted({q for q, _ in pairs})
    pos = {q: i for i, q in enumerate(measured)}
    dist = marginal(probs, circuit.num_qubits, measured)
    cum = np.cumsum(dist)
    cum /= cum[-1]
    idx = np.minimum(np.searchsorted(cum, rng.random(shots), side="right").astype(np.int64), len(dist) - 1)
    wide = circuit.num_clbits > 62
    bits = np.zeros(shots, dtype=object if wide else np.int64)
    for q, c in pairs:
        val = (idx >> pos[q]) & 1
        err = noise.readout_error(q) if noise else None
        if err is not None and (err.p01 or err.p10):
            val = val ^ (rng.random(shots) < np.where(val == 1, err.p10, err.p01)).astype(np.int64)
        if wide:
            bits = bits + np.array([int(v) << c for v in val], dtype=object)
        else:
            bits |= val << c
    keys, counts = np.unique(bits, return_counts=True)
    return {circuit.format_bits(int(k)): int(m) for k, m in zip(keys, counts, strict=True)}


# ----------------------------------------------------------------------- trajectories


def traj_channel(v: C128, n: int, ch: Any, qubits: tuple[int, ...], rng: np.random.Generator) -> C128:
    """One Kraus branch with its Born weight; always one uniform (``engines.py:159-183``)."""
    r = rng.random()
    if ch.mixture is not None:
        acc = 0.0
        for p, u in ch.mixture:
            acc += p
            if r < acc:
                if not np.allclose(u, np.eye(u.shape[0])):
                    v = apply_bits(v, n, u, list(qubits))
                return v
        return v
    acc = 0.0
    cand = v
    for k in ch.kraus:
        cand = apply_bits(v, n, k, list(qubits))
        w = float(np.vdot(cand, cand).real)
        acc += w
        if r < acc and w > 0:
            return cand / np.sqrt(w)
    w = float(np.vdot(cand, cand).real)
    return cand / np.sqrt(w) if w > 0 else v


def traj_measure(v: C128, n: int, q: int, rng: np.random.Generator) -> tuple[C128, int]:
    """``engines.py:185-201``: p1 clipped, outcome by one uniform, collapse and renormalise."""
    one = v.reshape(-1, 2, 1 << q)[:, 1, :]
    p1 = min(max(float(np.vdot(one, one).real), 0.0), 1.0)
    outcome = int(rng.random() < p1)
    prob = p1 if outcome else 1 - p1
    w = v.reshape(-1, 2, 1 << q).copy()
    w[:, 1 - outcome, :] = 0
    w = w.reshape(-1)
    if prob > 0:
        w = w / np.sqrt(prob)
    return w, outcome


def trajectory(circuit: Any, noise: Any, rng: np.random.Generator) -> int:
    """One shot (``simulator.py:287-317``); returns the classical bits as an integer."""
    n = circuit.num_qubits
    state = [sv_zero(n)]
    clbits = [0] * circuit.num_clbits

    def walk(ops: Any) -> None:
        for op in ops:
            k = op.kind
            if k == "gate":
                state[0] = apply_bits(state[0], n, op.matrix, list(op.qubits))
                ch = noise.gate_error(op.name, op.qubits) if noise else None
                if ch is not None:
                    state[0] = traj_channel(state[0], n, ch, op.qubits, rng)
            elif k == "measure":
                state[0], out = traj_measure(state[0], n, op.qubit, rng)
                err = noise.readout_error(op.qubit) if noise else None
                if err is not None and rng.random() < (err.p10 if out else err.p01):
                    out ^= 1
                if op.clbit is not None:
                    clbits[op.clbit] = out
            elif k == "reset":
                state[0], out = traj_measure(state[0], n, op.qubit, rng)
                if out:
                    state[0] = apply_bits(state[0], n, X, [op.qubit])
            elif k == "gphase":
                state[0] = state[0] * np.exp(1j * op.angle)
            elif k == "if":
                walk(op.then if op.condition.holds(clbits) else op.otherwise)

    walk(circuit.operations)
    return sum(b << i for i, b in enumerate(clbits))


def exact_outcomes(circuit: Any, noise: Any = None) -> dict[int, float]:
    """The exact distribution of the classical bits a trajectory run produces, for circuits with
    mid-circuit measurement, conditions and resets: one density matrix per classical record,
    summed over the shots' branches. The trajectory rules it averages are ``simulator.py:287-317``
    with ``engines.py:159-205``: a gate's noise channel picked by Born weight averages to the
    channel; a measurement splits a record by projection, its readout error mixes the recorded
    bit; a reset (measure, then X on 1) is the channel {|0><0|, |0><1|}; a condition picks the
    branch per record. Keys are the classical bits as an integer (bit c = classical bit c)."""
    n = circuit.num_qubits
    if n > 10:
        raise OracleError("exact trajectory outcomes are for up to 10 qubits")
    nb = 2 * n
    rho0 = np.zeros(1 << nb, dtype=np.complex128)
    rho0[0] = 1
    records: dict[tuple[int, ...], C128] = {tuple([0] * circuit.num_clbits): rho0}
    reset_kraus = (np.array([[1, 0], [0, 0]], dtype=np.complex128), np.array([[0, 1], [0, 0]], dtype=np.complex128))

    def project(rho: C128, q: int, bit: int) -> C128:
        proj = np.diag([1.0 - bit, float(bit)]).astype(np.complex128)
        return apply_bits(apply_bits(rho, nb, proj, [n + q]), nb, proj, [q])

    def walk(recs: dict[tuple[int, ...], C128], ops: Any) -> dict[tuple[int, ...], C128]:
        for op in ops:
            k = op.kind
            if k == "gate":
                ch = noise.gate_error(op.name, op.qubits) if noise else None
                for key, rho in recs.items():
                    rho = apply_bits(rho, nb, op.matrix, [n + q for q in op.qubits])
                    rho = apply_bits(rho, nb, op.matrix.conj(), list(op.qubits))
                    recs[key] = dm_channel(rho, n, ch, op.qubits) if ch is not None else rho
            elif k == "measure":
                err = noise.readout_error(op.qubit) if noise else None
                p01, p10 = (float(err.p01), float(err.p10)) if err is not None else (0.0, 0.0)
                out: dict[tuple[int, ...], C128] = {}
                for key, rho in recs.items():
                    for true in (0, 1):
                        part = project(rho, op.qubit, true)
                        flip = p10 if true else p01
                        for seen, w in ((true, 1.0 - flip), (true ^ 1, flip)):
                            if w == 0.0:
                                continue
                            bits = list(key)
                            if op.clbit is not None:
                                bits[op.clbit] = seen
                            t = tuple(bits)
                            out[t] = out[t] + w * part if t in out else w * part
                recs = out
            elif k == "reset":
                for key, rho in recs.items():
                    recs[key] = dm_kraus(rho, n, reset_kraus, (op.qubit,))
            elif k == "if":
                yes = {kk: v for kk, v in recs.items() if op.condition.holds(list(kk))}
                no = {kk: v for kk, v in recs.items() if not op.condition.holds(list(kk))}
                recs = walk(yes, op.then)
                for kk, v in walk(no, op.otherwise).items():
                    recs[kk] = recs[kk] + v if kk in recs else v
        return recs

    final = walk(records, circuit.operations)
    d = 1 << n
    return {sum(b << i for i, b in enumerate(key)): float(np.real(np.trace(rho.reshape(d, d)))) for key, rho in final.items()}


# ----------------------------------------------------------------------------- run


def choose(circuit: Any, noise: Any, method: str) -> str:
    """Method choice (``simulator.py:157-193``) for the four native methods."""
    from oracle.clifford import clifford_problem

    gate_noise = noise is not None and noise.has_gate_errors()
    dynamic = circuit.is_dynamic()
    if method == "automatic":
        if circuit.num_qubits >= AUTO_STABILIZER_QUBITS and clifford_problem(circuit, noise) is None:
            return "stabilizer"
        if dynamic:
            return "trajectories"
        if gate_noise:
            return "density_matrix" if circuit.num_qubits <= AUTO_DENSITY_QUBITS else "trajectories"
        return "statevector"
    return method


def run_counts(circuit: Any, shots: int, seed: int | None, noise: Any = None, method: str = "automatic") -> tuple[dict[str, int], str, int]:  # noqa: E501
    """Counts as ``simulator.py:320-393`` produces them, plus the method and seed used."""
    from oracle import tableau

    chosen = choose(circuit, noise, method)
    seed = secrets.randbelow(2**63) if seed is None else int(seed)
    rng = np.random.default_rng(seed)
    if chosen == "stabilizer":
        tally = tableau.run_counts(circuit, shots, noise, rng)
        counts = {circuit.format_bits(b): m for b, m in sorted(tally.items())} if circuit.num_clbits else {}
    elif chosen == "trajectories":
        if circuit.num_qubits > MAX_STATEVECTOR_QUBITS:
            raise OracleError("too many qubits")
        t: dict[int, int] = {}
        for _ in range(shots):
            b = trajectory(circuit, noise, rng)
            t[b] = t.get(b, 0) + 1
        counts = {circuit.format_bits(b): m for b, m in sorted(t.items())} if circuit.num_clbits else {}
    elif chosen == "statevector":
        probs = np.abs(evolve_sv(circuit)) ** 2
        counts = sample(circuit, probs, shots, noise, rng)
    else:
        probs = dm_probabilities(evolve_dm(circuit, noise), circuit.num_qubits)
        counts = sample(circuit, probs, shots, noise, rng)
    return dict(sorted(counts.items())), chosen, seed


def probabilities_array(circuit: Any, noise: Any = None) -> NDArray[np.float64]:
    """Exact probabilities (``simulator.py:424-442``) as the full array."""
    if noise is not None and noise.has_gate_errors():
        return dm_probabilities(evolve_dm(circuit, noise), circuit.num_qubits)
    return np.abs(evolve_sv(circuit)) ** 2


def outcome_probabilities(circuit: Any, noise: Any = None, threshold: float = 1e-12) -> dict[str, float]:
    """Readout-error branching over measured outcomes (``simulator.py:445-486``)."""
    pairs = circuit.final_measurements()
    if not pairs:
        return {}
    probs = probabilities_array(circuit, noise)
    measured = sorted({q for q, _ in pairs})
    pos = {q: i for i, q in enumerate(measured)}
    dist = marginal(probs, circuit.num_qubits, measured)
    out: dict[int, float] = {}
    for index, p in enumerate(dist):
        if p <= threshold:
            continue
        branches = [(0, float(p))]
        for q, c in pairs:
            bit = (index >> pos[q]) & 1
            err = noise.readout_error(q) if noise else None
            flip = (err.p10 if bit else err.p01) if err is not None else 0.0
            nxt = []
            for b, w in branches:
                if flip < 1:
                    nxt.append((b | (bit << c), w * (1 - flip)))
                if flip > 0:
                    nxt.append((b | ((bit ^ 1) << c), w * flip))
            branches = nxt
        for b, w in branches:
            out[b] = out.get(b, 0.0) + w
    return {circuit.format_bits(b): w for b, w in sorted(out.items()) if w > threshold}


def pauli_masks(label: str) -> tuple[int, int]:
    """(x mask, z mask) of a Pauli label, qubit 0 rightmost; Y sets both."""
    xm = zm = 0
    for q, letter in enumerate(reversed(label.upper())):
        if letter in "XY":
            xm |= 1 << q
        if letter in "ZY":
            zm |= 1 << q
    return xm, zm


_PAULI = {
    "X": np.array([[0, 1], [1, 0]], dtype=np.complex128),
    "Y": np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    "Z": np.array([[1, 0], [0, -1]], dtype=np.complex128),
}


def expectation(circuit: Any, observable: Any, noise: Any = None) -> float:
    """Σ w ⟨P⟩ (``simulator.py:489-527``): ket copy with Paulis applied, or Pauli-left trace."""
    terms = {observable: 1.0} if isinstance(observable, str) else dict(observable)
    n = circuit.num_qubits
    total = 0.0
    if noise is not None and noise.has_gate_errors():
        rho = evolve_dm(circuit, noise)
        d = 1 << n
        for label, w in terms.items():
            probe = rho
            for q, letter in enumerate(reversed(label.upper())):
                if letter != "I":
                    probe = apply_bits(probe, 2 * n, _PAULI[letter], [n + q])
            total += w * float(np.trace(probe.reshape(d, d)).real)
        return total
    ket = evolve_sv(circuit)
    for label, w in terms.items():
        probe = ket.copy()
        for q, letter in enumerate(reversed(label.upper())):
            if letter != "I":
                probe = apply_bits(probe, n, _PAULI[letter], [q])
        total += w * float(np.vdot(ket, probe).real)
    return total
