"""Noise channels and the noise model, on the host.

The engine turns these into device work: Pauli mixtures become per-shot branch choices,
Kraus channels become superoperators on the vectorised density matrix. The rules here decide
*which* channel follows *which* gate and must agree with Orrery exactly, so they mirror
``src/lucivant_sim/noise.py``: branch order of Pauli channels (identity first, then labels sorted,
``noise.py:66-85``), the depolarising parameterisation (``:88-105``), thermal-relaxation Kraus
products (``:134-144``), and rule specificity with the last rule winning ties (``:169-178``,
``:219-225``). :meth:`NoiseModel.digest` hashes the same description as ``noise.py:230-249``.
"""

from __future__ import annotations

import hashlib
import itertools
import json
import math
from collections.abc import Iterable, Mapping, Sequence
from dataclasses import dataclass, field
from pathlib import Path
from typing import Any

import numpy as np

from lucivant_sim_gb300.gates import Matrix, canonical_name, pauli_string_matrix

#: Frame changes on real hardware: no default error attaches to them.
IDEAL_GATES = frozenset({"rz", "p", "phase", "u1", "id", "i", "u0"})


@dataclass(frozen=True, eq=False)
class Channel:
    """A CPTP map by its Kraus operators. ``mixture`` lists (probability, unitary) branches when
    the channel is a mix of unitaries; ``analytic_depolarizing`` allows the partial-trace form."""

    name: str
    num_qubits: int
    kraus: tuple[Matrix, ...]
    params: tuple[float, ...] = ()
    mixture: tuple[tuple[float, Matrix], ...] | None = None
    analytic_depolarizing: bool = False

    def __post_init__(self) -> None:
        d = 1 << self.num_qubits
        acc = np.zeros((d, d), dtype=np.complex128)
        for k in self.kraus:
            acc += k.conj().T @ k
        if not np.allclose(acc, np.eye(d), atol=1e-9):
            raise ValueError(f"{self.name}: the Kraus operators don't preserve probability")

    def describe(self) -> list[Any]:
        return [self.name, self.num_qubits, [round(p, 15) for p in self.params]]


def _checked(p: float, what: str, upper: float = 1.0) -> float:
    if math.isnan(p) or not 0.0 <= p <= upper:
        raise ValueError(f"{what} must be between 0 and {upper:g}, not {p}")
    return float(p)


def pauli_channel(probabilities: Mapping[str, float]) -> Channel:
    """Pauli string P with probability probabilities[P], identity with the rest."""
    width = len(next(iter(probabilities)))
    total = sum(probabilities.values())
    _checked(total, "the total Pauli probability")
    branches: list[tuple[float, Matrix]] = []
    if total < 1:
        branches.append((1 - total, np.eye(1 << width, dtype=np.complex128)))
    for label in sorted(probabilities):
        p = probabilities[label]
        if len(label) != width or set(label) - set("IXYZ"):
            raise ValueError(f"{label!r} isn't a {width}-qubit Pauli string")
        if p <= 0:
            continue
        branches.append((p, pauli_string_matrix(label)))
    kraus = tuple(math.sqrt(p) * m for p, m in branches)
    params = tuple(probabilities[label] for label in sorted(probabilities))
    return Channel("pauli", width, kraus, params, tuple(branches))


def depolarizing(p: float, num_qubits: int = 1) -> Channel:
    """Replace the state by the maximally mixed one with probability p (each non-identity
    Pauli with probability p/4**k)."""
    d2 = 4**num_qubits
    _checked(p, "a depolarising probability", d2 / (d2 - 1))
    probs = {
        "".join(letters): p / d2
        for letters in itertools.product("IXYZ", repeat=num_qubits)
        if set(letters) != {"I"}
    }
    base = pauli_channel(probs)
    return Channel("depolarizing", num_qubits, base.kraus, (p,), base.mixture, analytic_depolarizing=True)


class GateErrors:
    """:meth:`NoiseModel.gate_error` over many models at once (``None`` entries: no noise). Models
    sharing a rule shape share the winning rule's index, found once per gate signature, so a batch
    of noise instances of one template costs one rule search per gate instead of one per model."""

    def __init__(self, models: Sequence[NoiseModel | None]) -> None:
        self.models = list(models)
        shapes: dict[tuple[Any, ...], int] = {}
        self.shape_of = [None if m is None else shapes.setdefault(m.rule_shape(), len(shapes)) for m in self.models]
        self.first = {}
        for i, sh in enumerate(self.shape_of):
            if sh is not None:
                self.first.setdefault(sh, i)

    def __call__(self, name: str, qubits: tuple[int, ...]) -> list[Channel | None]:
        winner: dict[int, int] = {}
        for sh, i in self.first.items():
            best, best_score = -1, -1.0
            for j, rule in enumerate(self.models[i].rules):
                s = rule.score(name, qubits)
                if s >= 0 and s >= best_score:
                    best, best_score = j, s
            winner[sh] = best
        out: list[Channel | None] = []
        for m, sh in zip(self.models, self.shape_of):
            j = -1 if sh is None else winner[sh]
            out.append(None if j < 0 else m.rules[j].channel)  # type: ignore[union-attr]
        return out


def from_gate_error(error: float, num_qubits: int) -> Channel:
    """The depolarising channel with average gate infidelity ``error`` (p = r d/(d-1))."""
    d = 1 << num_qubits
    p = min(error * d / (d - 1), 4**num_qubits / (4**num_qubits - 1))
    return depolarizing(p, num_qubits)


def bit_flip(p: float) -> Channel:
    base = pauli_channel({"X": _checked(p, "a bit-flip probability")})
    return Channel("bit_flip", 1, base.kraus, (p,), base.mixture)


def phase_flip(p: float) -> Channel:
    base = pauli_channel({"Z": _checked(p, "a phase-flip probability")})
    return Channel("phase_flip", 1, base.kraus, (p,), base.mixture)


def amplitude_damping(gamma: float) -> Channel:
    g = _checked(gamma, "gamma")
    k0 = np.array([[1, 0], [0, math.sqrt(1 - g)]], dtype=np.complex128)
    k1 = np.array([[0, math.sqrt(g)], [0, 0]], dtype=np.complex128)
    return Channel("amplitude_damping", 1, (k0, k1), (g,))


def phase_damping(lam: float) -> Channel:
    lam = _checked(lam, "lambda")
    k0 = np.array([[1, 0], [0, math.sqrt(1 - lam)]], dtype=np.complex128)
    k1 = np.array([[0, 0], [0, math.sqrt(lam)]], dtype=np.complex128)
    return Channel("phase_damping", 1, (k0, k1), (lam,))


def thermal_relaxation(t1: float, t2: float, time: float) -> Channel:
    """T1 relaxation and T2 dephasing over ``time``: Kraus set {pd_j @ ad_i}."""
    if t1 <= 0 or t2 <= 0 or time < 0:
        raise ValueError("T1 and T2 must be positive and the time not negative")
    if t2 > 2 * t1 + 1e-12:
        raise ValueError("T2 can't exceed 2*T1")
    gamma = 1 - math.exp(-time / t1)
    lam = max(0.0, 1 - math.exp(-2 * time / t2 + time / t1))
    ad, pd = amplitude_damping(gamma), phase_damping(min(lam, 1.0))
    kraus = tuple(b @ a for a in ad.kraus for b in pd.kraus)
    return Channel("thermal_relaxation", 1, kraus, (t1, t2, time))


@dataclass(frozen=True)
class ReadoutError:
    """p01: read 1 for a 0; p10: read 0 for a 1."""

    p01: float
    p10: float

    def __post_init__(self) -> None:
        _checked(self.p01, "p01")
        _checked(self.p10, "p10")

    @classmethod
    def symmetric(cls, p: float) -> ReadoutError:
        return cls(p, p)


@dataclass
class _Rule:
    channel: Channel
    gates: frozenset[str] | None
    qubits: tuple[int, ...] | None

    def score(self, name: str, qubits: tuple[int, ...]) -> float:
        if self.channel.num_qubits != len(qubits):
            return -1
        if self.gates is not None and name not in self.gates:
            return -1
        if self.qubits is not None and sorted(self.qubits) != sorted(qubits):
            return -1
        if self.gates is None and name in IDEAL_GATES:
            return -1
        return (2 if self.qubits is not None else 0) + (1 if self.gates is not None else 0)


@dataclass
class NoiseModel:
    """Which channel follows which gate, and each qubit's readout error. The most specific rule
    wins; among equals, the one added last."""

    rules: list[_Rule] = field(default_factory=list)
    readout: dict[int | None, ReadoutError] = field(default_factory=dict)
    source: str | None = None

    def add_gate_error(
        self,
        channel: Channel,
        gates: str | Iterable[str] | None = None,
        qubits: Sequence[int] | None = None,
    ) -> NoiseModel:
        names = None
        if gates is not None:
            names = frozenset(canonical_name(g) for g in ([gates] if isinstance(gates, str) else gates))
        if qubits is not None and len(qubits) != channel.num_qubits:
            raise ValueError(f"a {channel.num_qubits}-qubit channel can't attach to {len(qubits)} qubit(s)")
        self.rules.append(_Rule(channel, names, tuple(qubits) if qubits is not None else None))
        return self

    def add_readout_error(self, error: float | ReadoutError, qubits: Iterable[int] | None = None) -> NoiseModel:
        err = error if isinstance(error, ReadoutError) else ReadoutError.symmetric(float(error))
        for q in [None] if qubits is None else qubits:
            self.readout[q] = err
        return self

    def gate_error(self, name: str, qubits: tuple[int, ...]) -> Channel | None:
        best, best_score = None, -1.0
        for rule in self.rules:
            s = rule.score(name, qubits)
            if s >= 0 and s >= best_score:
                best, best_score = rule.channel, s
        return best

    def rule_shape(self) -> tuple[Any, ...]:
        """What rule selection reads (each rule's gates, qubits and channel width, in order): models
        of one shape pick the same rule for every gate."""
        return tuple((r.gates, r.qubits, r.channel.num_qubits) for r in self.rules)

    def readout_error(self, qubit: int) -> ReadoutError | None:
        return self.readout.get(qubit, self.readout.get(None))

    def has_gate_errors(self) -> bool:
        return bool(self.rules)

    def is_empty(self) -> bool:
        return not self.rules and not any(e.p01 or e.p10 for e in self.readout.values())

    def describe(self) -> dict[str, Any]:
        return {
            "rules": [
                [sorted(r.gates) if r.gates is not None else None, list(r.qubits or []) or None, r.channel.describe()]
                for r in self.rules
            ],
            "readout": sorted(
                [[-1 if q is None else q, round(e.p01, 15), round(e.p10, 15)] for q, e in self.readout.items()]
            ),
        }

    def digest(self) -> str:
        text = json.dumps(self.describe(), separators=(",", ":"), sort_keys=True).encode()
        return "sha256:" + hashlib.sha256(text).hexdigest()

    @classmethod
    def uniform(cls, single: float = 0.0, two: float = 0.0, readout: float = 0.0) -> NoiseModel:
        model = cls(source="uniform")
        if single > 0:
            model.add_gate_error(from_gate_error(single, 1))
        if two > 0:
            model.add_gate_error(from_gate_error(two, 2))
        if readout > 0:
            model.add_readout_error(readout)
        return model

    @classmethod
    def from_calibration(cls, calibration: Mapping[str, Any] | str | Path) -> NoiseModel:
        """Medians plus per-qubit and per-coupler errors from a twin-format calibration."""
        if isinstance(calibration, (str, Path)):
            cal: dict[str, Any] = json.loads(Path(calibration).read_text(encoding="utf-8"))
        else:
            cal = dict(calibration)
        if isinstance(cal.get("calibration"), Mapping):
            cal = dict(cal["calibration"])
        model = cls(source=str(cal.get("device") or cal.get("profile_key") or "calibration"))
        if cal.get("single_qubit_error"):
            model.add_gate_error(from_gate_error(float(cal["single_qubit_error"]), 1))
        if cal.get("two_qubit_error"):
            model.add_gate_error(from_gate_error(float(cal["two_qubit_error"]), 2))
        if cal.get("readout_error"):
            model.add_readout_error(float(cal["readout_error"]))
        for row in cal.get("qubits") or []:
            q = int(row["qubit"])
            if row.get("single_qubit_error") is not None:
                model.add_gate_error(from_gate_error(float(row["single_qubit_error"]), 1), qubits=[q])
            if row.get("readout_error") is not None:
                model.add_readout_error(float(row["readout_error"]), qubits=[q])
        for row in cal.get("couplers") or []:
            if row.get("error") is not None:
                a, b = (int(v) for v in row["qubits"])
                model.add_gate_error(from_gate_error(float(row["error"]), 2), qubits=[a, b])
        return model
