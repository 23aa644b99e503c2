"""Seeded synthetic circuits for the five benchmark workloads.

Every builder returns OpenQASM 3 text (angles written with ``repr(float)``, so parsing round-trips
exactly) and, for the very wide Clifford workload, can also build the Circuit directly, because
its text is tens of megabytes.

* brickwork(n, layers, seed): each layer applies u3(θ, φ, λ) to every qubit, θ, φ, λ i.i.d.
  uniform on [0, 2π) from ``default_rng(seed)`` drawn as one (layers, n, 3) array; then cx on
  (2i, 2i+1) in even layers and (2i+1, 2i+2) in odd layers.
* midcircuit(n, rounds, seed): each round is u3 on all qubits, brickwork cx, measure q[0..3]
  into c, ``if (c[k] == 1) x q[k+4]``, reset q[0..3]; finally q[4..7] are measured into f.
* clifford_layers(n, layers, seed): per qubit one of h/s/sdg/x/z uniformly, then a random
  perfect matching (``rng.permutation``) with cx then cz on each pair (a, b).
* hea(n, layers, seed): ry and rz layers with a linear cx chain (hardware-efficient ansatz).
"""

from __future__ import annotations

import math

import numpy as np

from lucivant_sim_gb300.circuit import ColumnarCircuit, Register
from lucivant_sim_gb300.gates import GATES
from lucivant_sim_gb300.noise import NoiseModel, ReadoutError, depolarizing, thermal_relaxation

TWO_PI = 2 * math.pi


def _header(n: int) -> list[str]:
    return ["OPENQASM 3.0;", 'include "stdgates.inc";', f"qubit[{n}] q;"]


def brickwork(n: int, layers: int, seed: int = 7, measure: bool = True) -> str:
    rng = np.random.default_rng(seed)
    angles = rng.uniform(0.0, TWO_PI, size=(layers, n, 3))
    lines = _header(n)
    if measure:
        lines.append(f"bit[{n}] c;")
    for layer in range(layers):
        for q in range(n):
            t, p, lam = (repr(float(v)) for v in angles[layer, q])
            lines.append(f"u3({t}, {p}, {lam}) q[{q}];")
        for a in range(layer % 2, n - 1, 2):
            lines.append(f"cx q[{a}], q[{a + 1}];")
    if measure:
        lines.append("c = measure q;")
    return "\n".join(lines) + "\n"


def midcircuit(n: int, rounds: int, seed: int = 7) -> str:
    if n < 8:
        raise ValueError("the mid-circuit workload needs at least 8 qubits")
    rng = np.random.default_rng(seed)
    angles = rng.uniform(0.0, TWO_PI, size=(rounds, n, 3))
    lines = _header(n) + ["bit[4] c;", "bit[4] f;"]
    for r in range(rounds):
        for q in range(n):
            t, p, lam = (repr(float(v)) for v in angles[r, q])
            lines.append(f"u3({t}, {p}, {lam}) q[{q}];")
        for a in range(r % 2, n - 1, 2):
            lines.append(f"cx q[{a}], q[{a + 1}];")
        for k in range(4):
            lines.append(f"c[{k}] = measure q[{k}];")
        for k in range(4):
            lines.append(f"if (c[{k}] == 1) x q[{k + 4}];")
        for k in range(4):
            lines.append(f"reset q[{k}];")
    lines.append("f = measure q[4:7];")
    return "\n".join(lines) + "\n"


_CLIFFORD_1Q = ("h", "s", "sdg", "x", "z")


def _clifford_plan(n: int, layers: int, seed: int) -> list[tuple[np.ndarray, np.ndarray]]:
    rng = np.random.default_rng(seed)
    plan = []
    for _ in range(layers):
        picks = rng.integers(0, len(_CLIFFORD_1Q), size=n)
        perm = rng.permutation(n)
        plan.append((picks, perm))
    return plan


def clifford_layers(n: int, layers: int, seed: int = 11) -> str:
    lines = _header(n) + [f"bit[{n}] c;"]
    for picks, perm in _clifford_plan(n, layers, seed):
        lines += [f"{_CLIFFORD_1Q[int(g)]} q[{q}];" for q, g in enumerate(picks)]
        for i in range(0, n - 1, 2):
            a, b = int(perm[i]), int(perm[i + 1])
            lines.append(f"cx q[{a}], q[{b}];")
            lines.append(f"cz q[{a}], q[{b}];")
    lines.append("c = measure q;")
    return "\n".join(lines) + "\n"


def clifford_layers_circuit(n: int, layers: int, seed: int = 11) -> ColumnarCircuit:
    """The same circuit as :func:`clifford_layers` without writing and parsing its text, held as
    arrays (a columnar circuit: its 4 million gates at 2048 qubits x 1000 layers need no per-gate
    objects for a stabilizer run)."""
    names = [*_CLIFFORD_1Q, "cx", "cz"]
    mats = [GATES[name].build() for name in names]
    cx, cz = len(_CLIFFORD_1Q), len(_CLIFFORD_1Q) + 1
    kinds, rows, arity = [], [], []
    for picks, perm in _clifford_plan(n, layers, seed):
        pairs = n // 2
        a, b = perm[0 : 2 * pairs : 2], perm[1 : 2 * pairs : 2]
        kinds += [picks.astype(np.int64), np.tile(np.array([cx, cz], dtype=np.int64), pairs)]
        one = np.full((n, 3), -1, dtype=np.int64)
        one[:, 0] = np.arange(n)
        two = np.full((2 * pairs, 3), -1, dtype=np.int64)
        two[:, 0], two[:, 1] = np.repeat(a, 2), np.repeat(b, 2)
        rows += [one, two]
        arity += [np.ones(n, dtype=np.int64), np.full(2 * pairs, 2, dtype=np.int64)]
    kind = np.concatenate(kinds) if kinds else np.zeros(0, dtype=np.int64)
    qubits = np.concatenate(rows) if rows else np.zeros((0, 3), dtype=np.int64)
    ar = np.concatenate(arity) if arity else np.zeros(0, dtype=np.int64)
    return ColumnarCircuit(n, n, names, mats, kind, qubits, ar, [(q, q) for q in range(n)],
                           (Register("q", 0, n),), (Register("c", 0, n),))  # fmt: skip


def hea(n: int, layers: int, seed: int, measure: bool = False) -> str:
    rng = np.random.default_rng(seed)
    angles = rng.uniform(0.0, TWO_PI, size=(layers, n, 2))
    lines = _header(n)
    if measure:
        lines.append(f"bit[{n}] c;")
    for layer in range(layers):
        for q in range(n):
            lines.append(f"ry({float(angles[layer, q, 0])!r}) q[{q}];")
            lines.append(f"rz({float(angles[layer, q, 1])!r}) q[{q}];")
        for a in range(n - 1):
            lines.append(f"cx q[{a}], q[{a + 1}];")
    if measure:
        lines.append("c = measure q;")
    return "\n".join(lines) + "\n"


def random_pauli_sum(n: int, terms: int, seed: int) -> dict[str, float]:
    """``terms`` random Pauli strings (qubit 0 rightmost) with N(0, 1) coefficients."""
    rng = np.random.default_rng(seed)
    out: dict[str, float] = {}
    while len(out) < terms:
        label = "".join("IXYZ"[int(v)] for v in rng.integers(0, 4, size=n))
        out[label] = out.get(label, 0.0) + float(rng.normal())
    return out


def dm_noise(single: float = 1e-3, two: float = 1e-2, readout: float = 2e-2) -> NoiseModel:
    """Uniform gate and readout noise, with thermal relaxation (T1 = 120, T2 = 90, t = 0.05)
    on u3. By the rule-specificity order, thermal relaxation replaces the uniform one-qubit
    error on u3 (a gate-named rule outranks a gate-agnostic one)."""
    return NoiseModel.uniform(single=single, two=two, readout=readout).add_gate_error(
        thermal_relaxation(t1=120, t2=90, time=0.05), gates="u3"
    )


def stabilizer_noise(p: float = 1e-3) -> NoiseModel:
    """Depolarising p on every one- and two-qubit gate, readout p01 = 0.01, p10 = 0.03."""
    model = NoiseModel()
    model.add_gate_error(depolarizing(p, 1))
    model.add_gate_error(depolarizing(p, 2))
    model.add_readout_error(ReadoutError(0.01, 0.03))
    return model


def thermal_depolarizing(single: float, t1: float = 120, t2: float = 90, time: float = 0.05):
    """Depolarising error of average infidelity ``single`` followed by thermal relaxation, as one
    Kraus channel (products T_j @ D_i): the reading of "uniform noise plus thermal relaxation on
    every u3" in which both act, so the one-qubit error parameter matters."""
    from lucivant_sim_gb300.noise import Channel, from_gate_error

    th = thermal_relaxation(t1, t2, time)
    dp = from_gate_error(single, 1)
    kraus = tuple(t @ d for d in dp.kraus for t in th.kraus)
    return Channel("thermal_relaxation+depolarizing", 1, kraus, (t1, t2, time, dp.params[0]))


def dm_noise_instances(count: int, seed: int = 7, readout: float = 2e-2) -> list[NoiseModel]:
    """``count`` noise instances: one-qubit error uniform in [1e-4, 5e-3] and two-qubit error
    uniform in [1e-3, 3e-2], seeded; thermal relaxation composed with the one-qubit error on u3."""
    rng = np.random.default_rng(seed)
    singles = rng.uniform(1e-4, 5e-3, size=count)
    twos = rng.uniform(1e-3, 3e-2, size=count)
    return [
        NoiseModel.uniform(two=float(t), readout=readout).add_gate_error(thermal_depolarizing(float(s)), gates="u3")
        for s, t in zip(singles, twos, strict=True)
    ]


def z_observables(n: int) -> list[str]:
    """<Z_i> for every qubit and <Z_i Z_{i+1}> for neighbours (qubit 0 rightmost)."""
    labels = []
    for i in range(n):
        lab = ["I"] * n
        lab[n - 1 - i] = "Z"
        labels.append("".join(lab))
    for i in range(n - 1):
        lab = ["I"] * n
        lab[n - 1 - i] = "Z"
        lab[n - 2 - i] = "Z"
        labels.append("".join(lab))
    return labels


def hea_template(n: int, layers: int) -> str:
    """A hardware-efficient ansatz with one ``input float`` per rotation (p0, p1, ...): ry and rz
    on every qubit per layer, then a linear cx chain."""
    names = [f"p{i}" for i in range(2 * n * layers)]
    lines = ["OPENQASM 3.0;", 'include "stdgates.inc";'] + [f"input float {v};" for v in names] + [f"qubit[{n}] q;"]
    k = 0
    for _layer in range(layers):
        for q in range(n):
            lines.append(f"ry({names[k]}) q[{q}];")
            lines.append(f"rz({names[k + 1]}) q[{q}];")
            k += 2
        for a in range(n - 1):
            lines.append(f"cx q[{a}], q[{a + 1}];")
    return "\n".join(lines) + "\n"


def served_mix(jobs: int = 2000, rate: float = 200.0, seed: int = 5, shots: int = 1000, sweep: int = 8,
               widths: tuple[int, int] = (8, 26), depths: tuple[int, int] = (10, 100)) -> list[dict]:  # fmt: skip
    """The served mix: Poisson arrivals at ``rate`` jobs/s; widths uniform over ``widths`` (8..26)
    and depths over ``depths`` (10..100), u3+cx brickwork. 30% are hardware-efficient-ansatz sweeps (``sweep`` parameter
    sets of one template, angles U[0, 2π)) measured on a 20-term random Pauli sum with N(0, 1)
    coefficients; 20% carry uniform noise (1e-3, 1e-2, readout 2e-2) on the density-matrix path
    at the three smallest widths (8..10); the rest are sampled with ``shots`` shots. Every job is OpenQASM text."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=jobs))
    out = []
    for i in range(jobs):
        u = rng.uniform()
        depth = int(rng.integers(depths[0], depths[1] + 1))
        job_seed = int(rng.integers(0, 2**31))
        if u < 0.3:
            n = int(rng.integers(widths[0], widths[1] + 1))
            layers = max(1, depth // 10)
            params = [dict(zip([f"p{k}" for k in range(2 * n * layers)],
                               np.random.default_rng(job_seed + s).uniform(0, TWO_PI, size=2 * n * layers).tolist()))
                      for s in range(sweep)]  # fmt: skip
            out.append(dict(kind="expect", arrival=float(arrivals[i]), qasm=hea_template(n, layers), params=params,
                            observable=random_pauli_sum(n, 20, job_seed), width=n, depth=layers))
        elif u < 0.5:
            n = int(rng.integers(widths[0], min(widths[0] + 2, widths[1]) + 1))
            out.append(dict(kind="density", arrival=float(arrivals[i]), qasm=brickwork(n, depth, seed=job_seed),
                            shots=shots, seed=job_seed, width=n, depth=depth))
        else:
            n = int(rng.integers(widths[0], widths[1] + 1))
            out.append(dict(kind="sample", arrival=float(arrivals[i]), qasm=brickwork(n, depth, seed=job_seed),
                            shots=shots, seed=job_seed, width=n, depth=depth))
    return out
