"""The public API with Orrery's signatures and semantics, running on the GB300 engine.

``run``, ``statevector``, ``density_matrix``, ``probabilities``, ``outcome_probabilities``,
``expectation`` and ``verify`` take and return what ``src/lucivant_sim/simulator.py:320-547``
does; method choice (``:157-193``), seeding (one PCG64 ``default_rng(seed)`` per run, ``:342-345``),
the order every uniform is drawn in, digests and the ``Result`` record are the same. The heavy
steps run on the GPU; the host draws the uniforms from NumPy's generator (or the device
regenerates the same PCG64 stream), so counts match Orrery's for the same seed. A result records
the engine in ``version`` (``0.3.0+gb300-N``), as Orrery's accelerator methods do
(``simulator.py:349-360``).
"""

from __future__ import annotations

import hashlib
import json
import os
import secrets
import time
from collections.abc import Mapping
from dataclasses import dataclass, field
from pathlib import Path
from typing import Any

import numpy as np
from numpy.typing import NDArray

from lucivant_sim_gb300 import _lib, engine
from lucivant_sim_gb300.circuit import Circuit, ColumnarCircuit, final_measurements, format_bits, format_bits_bytes
from lucivant_sim_gb300.clifford import clifford_problem
from lucivant_sim_gb300.engine import MAX_DENSITY_QUBITS, SimulationError, pauli_masks
from lucivant_sim_gb300.qasm import load, parse

__version__ = "0.3.0"
ENGINE = "gb300"

METHODS: tuple[str, ...] = (
    "automatic",
    "statevector",
    "density_matrix",
    "trajectories",
    "stabilizer",
    "statevector_aer",
    "stabilizer_stim",
)
AUTO_DENSITY_QUBITS = 10
AUTO_STABILIZER_QUBITS = 12
MAX_SHOTS = 10_000_000


def engine_version() -> str:
    return f"{__version__}+{ENGINE}-{_lib.library().lsg_version()}"


def to_circuit(program: Any, params: Mapping[str, float] | None = None) -> Any:
    """A circuit from OpenQASM text, a .qasm path, or an already-built circuit (this package's or
    Orrery's own: both are read through their ``kind``-tagged operations)."""
    if isinstance(program, os.PathLike):
        return load(Path(program), params)
    if isinstance(program, str):
        return parse(program, params)
    # a columnar circuit builds its operation objects only when asked: never just to recognise it
    if isinstance(program, (Circuit, ColumnarCircuit)) or (hasattr(program, "operations") and hasattr(program, "num_qubits")):
        if params:
            raise ValueError("params apply to OpenQASM source, not to an already-built Circuit")
        return program
    raise TypeError(f"can't simulate a {type(program).__name__}; give OpenQASM, a path, or a Circuit")


def _digest(data: Any) -> str:
    return "sha256:" + hashlib.sha256(json.dumps(data, separators=(",", ":"), sort_keys=True).encode()).hexdigest()


@dataclass(frozen=True)
class Result:
    counts: dict[str, int]
    shots: int
    seed: int
    method: str
    num_qubits: int
    num_clbits: int
    circuit_digest: str
    noise_digest: str | None
    version: str
    elapsed_seconds: float
    statevector: NDArray[np.complex128] | None = field(default=None, repr=False, compare=False)
    #: Engine report: shots whose uniform fell within 1e-12 of a CDF boundary (the only shots a
    #: different floating-point summation order could move), and similar diagnostics.
    report: dict[str, Any] = field(default_factory=dict, repr=False, compare=False)

    @property
    def fingerprint(self) -> str:
        return _digest(
            {
                "engine": "lucivant-sim",
                "version": self.version,
                "circuit": self.circuit_digest,
                "noise": self.noise_digest,
                "shots": self.shots,
                "seed": self.seed,
                "method": self.method,
            }
        )

    @property
    def counts_digest(self) -> str:
        return _digest(self.counts)

    def frequencies(self) -> dict[str, float]:
        return {k: v / self.shots for k, v in self.counts.items()} if self.shots else {}

    def most_frequent(self) -> str | None:
        return max(self.counts, key=lambda k: (self.counts[k], k)) if self.counts else None

    def to_dict(self) -> dict[str, Any]:
        return {
            "engine": "lucivant-sim",
            "version": self.version,
            "method": self.method,
            "shots": self.shots,
            "seed": self.seed,
            "num_qubits": self.num_qubits,
            "num_clbits": self.num_clbits,
            "counts": self.counts,
            "circuit_digest": self.circuit_digest,
            "noise_digest": self.noise_digest,
            "fingerprint": self.fingerprint,
            "counts_digest": self.counts_digest,
            "elapsed_seconds": self.elapsed_seconds,
        }


def choose_method(circuit: Any, noise: Any, method: str = "automatic") -> str:
    """``simulator.py:157-193``, with the same messages."""
    if method not in METHODS:
        raise ValueError(f"method must be one of {', '.join(METHODS)}")
    gate_noise = noise is not None and noise.has_gate_errors()
    dynamic = circuit.is_dynamic() if hasattr(circuit, "is_dynamic") else False
    if method == "automatic":
        if circuit.num_qubits >= AUTO_STABILIZER_QUBITS and clifford_problem(circuit, noise) is None:
            return "stabilizer"
        if dynamic:
            return "trajectories"
        if gate_noise:
            return "density_matrix" if circuit.num_qubits <= AUTO_DENSITY_QUBITS else "trajectories"
        return "statevector"
    if method == "stabilizer":
        problem = clifford_problem(circuit, noise)
        if problem:
            raise SimulationError(f"the stabilizer method runs Clifford circuits only: {problem}")
        return method
    if method == "stabilizer_stim":
        if noise is not None and not noise.is_empty():
            raise SimulationError("stabilizer_stim runs ideal circuits; use 'stabilizer' for Pauli noise")
        if any(op.kind == "if" for op in circuit.operations):
            raise SimulationError("stabilizer_stim runs circuits without classical conditions; use 'stabilizer'")
        problem = clifford_problem(circuit, None)
        if problem:
            raise SimulationError(f"the stabilizer methods run Clifford circuits only: {problem}")
        return method
    if method in ("statevector", "statevector_aer") and (gate_noise or dynamic):
        raise SimulationError(
            "the statevector method runs ideal circuits without mid-circuit measurement; "
            "use 'density_matrix' or 'trajectories'"
        )
    if method == "density_matrix" and dynamic:
        raise SimulationError("this circuit uses measurement results mid-circuit; use 'trajectories'")
    if method == "density_matrix" and circuit.num_qubits > MAX_DENSITY_QUBITS:
        raise SimulationError(f"the density-matrix method handles up to {MAX_DENSITY_QUBITS} qubits")
    return method


# Orrery's accelerator methods and the package each runs on (``accel.py:45-51``)
_ACCELERATORS = {"statevector_aer": ("qiskit_aer", "Qiskit Aer"), "stabilizer_stim": ("stim", "Stim")}


def refuse_accelerator(method: str) -> None:
    """Orrery runs ``statevector_aer`` and ``stabilizer_stim`` on another package once the method
    is chosen and the seed checked (``simulator.py:339-357``); this engine has no path to them.
    Without the package the refusal is Orrery's own message; with it, the method is refused by
    name."""
    module, extra = _ACCELERATORS[method]
    try:
        __import__(module)
    except ImportError as exc:
        raise SimulationError(f"this method needs {extra}: pip install lucivant-sim[accel]") from exc
    raise SimulationError(f"the GB300 engine does not drive {extra}; use '{method.split('_')[0]}'")


def sample_register(
    reg: _lib.Register, circuit: Any, dm_qubits: int, shots: int, noise: Any, rng: np.random.Generator, member: int = 0
) -> tuple[dict[str, int], dict[str, Any]]:
    """``_sample`` (``simulator.py:254-284``) on the device: the host draws the uniforms in the
    reference's order — the CDF uniforms first, then one vector per measured pair with a readout
    error — and the device does the marginal, CDF, search and readout flips."""
    pairs = final_measurements(circuit)
    if not pairs or shots == 0:
        return {}, {"near_boundary": 0}
    measured = sorted({q for q, _ in pairs})
    position = {q: i for i, q in enumerate(measured)}
    uniforms = rng.random(shots)
    errs: list[tuple[float, float] | None] = []
    flips: list[np.ndarray] = []
    for q, _c in pairs:
        err = noise.readout_error(q) if noise else None
        if err is not None and (err.p01 or err.p10):
            errs.append((float(err.p01), float(err.p10)))
            flips.append(rng.random(shots))
        else:
            errs.append(None)
    flip_arr = np.concatenate(flips) if flips else None
    bits, near, near_count = reg.sample(dm_qubits, measured, uniforms, [position[q] for q, _ in pairs], errs, flip_arr,
                                        member)  # fmt: skip
    counts = count_bits(circuit, bits, [c for _, c in pairs])
    report = {"near_boundary": near_count}
    if near_count:
        report["near_boundary_shots"] = np.flatnonzero(near).tolist()
    return counts, report


def count_bits(circuit: Any, bits: np.ndarray, clbits: list[int]) -> dict[str, int]:
    """Pack per-pair outcome bits onto their classical bits and count (``simulator.py:279-284``);
    the result is ordered by outcome string, as :class:`Result` keeps its counts."""
    shots = bits.shape[0]
    if circuit.num_clbits > 62:
        keys = [sum(int(bits[s, j]) << c for j, c in enumerate(clbits)) for s in range(shots)]
        values, counts = np.unique(np.array(keys, dtype=object), return_counts=True)
        return dict(sorted((format_bits(circuit, int(v)), int(n)) for v, n in zip(values, counts, strict=True)))
    packed = np.zeros(shots, dtype=np.int64)
    for j, c in enumerate(clbits):
        packed |= bits[:, j].astype(np.int64) << c
    values, counts = np.unique(packed, return_counts=True)
    text = format_bits_bytes(circuit, values)
    # ASCII byte order is str order; numeric order is already string order for contiguous
    # registers (then the stable sort is a single pass)
    order = np.argsort(text, kind="stable")
    return dict(zip([b.decode() for b in text[order]], counts[order].tolist(), strict=True))


def _evolved(circuit: Any, noise: Any, precision: int) -> tuple[_lib.Register, int]:
    """The final static state on the device: statevector if ideal, density matrix if gate noise."""
    n = circuit.num_qubits
    if noise is not None and noise.has_gate_errors():
        return engine.evolve_density(circuit, [noise], precision), n
    reg = engine.new_statevector(n, precision)
    reg.apply_from_basis(engine.sv_oplist(circuit, fuse=True))
    return reg, 0


def precision_report(program: Any, noise: Any = None, observable: str | Mapping[str, float] | None = None,
                     params: Mapping[str, float] | None = None) -> dict[str, Any]:  # fmt: skip
    """How far the complex64 path's answers are from FP64 ones for a static circuit: the final
    state evolved on the device in complex64 (real32 for a density matrix in Pauli-transfer form)
    and again in complex128 (real64), compared.

    Returns ``max_amplitude_error`` (max |a64 - a128| over the statevector's amplitudes or the
    density matrix's entries; None for density matrices above 10 qubits, whose 4^n entries are not
    downloaded), ``probability_tvd`` (total-variation distance of the exact probabilities) and
    ``expectation_error`` (|<O>64 - <O>128| for ``observable``; without one, the largest error of
    the single-qubit <Z_q>)."""
    circuit = to_circuit(program, params)
    _static(circuit, "a precision report")
    n = circuit.num_qubits
    if observable is None:
        terms = {"".join("Z" if i == n - 1 - q else "I" for i in range(n)): 1.0 for q in range(n)}
        per_term = True
    else:
        terms = {observable: 1.0} if isinstance(observable, str) else dict(observable)
        per_term = False
    masks = [pauli_masks(label) for label in terms]
    weights = np.asarray(list(terms.values()))
    out: dict[str, Any] = {"reference": "complex128 re-run on the device"}
    states, probs, vals = [], [], []
    for prec in (_lib.C64, _lib.C128):
        reg, dm = _evolved(circuit, noise, prec)
        with reg:
            probs.append(reg.probabilities(dm))
            v = reg.expect(dm, [m[0] for m in masks], [m[1] for m in masks])[:, 0] if masks else np.zeros(0)
            vals.append(v if per_term else np.array([float(weights @ v)]))
            if dm == 0:
                states.append(reg.download()[0].astype(np.complex128))
            elif n <= 10:
                states.append(engine.density_download(reg))
    out["max_amplitude_error"] = float(np.max(np.abs(states[0] - states[1]))) if len(states) == 2 else None
    out["probability_tvd"] = 0.5 * float(np.abs(probs[0] - probs[1]).sum())
    out["expectation_error"] = float(np.max(np.abs(vals[0] - vals[1]))) if vals[0].size else 0.0
    out["form"] = "statevector" if not (noise is not None and noise.has_gate_errors()) else "density_matrix"
    return out


def run(
    program: Any,
    shots: int = 1024,
    *,
    seed: int | None = None,
    noise: Any = None,
    method: str = "automatic",
    params: Mapping[str, float] | None = None,
    precision: str | None = None,
    trajectory_mode: str | None = None,
    report_precision: bool = False,
) -> Result:
    """Simulate ``program`` ``shots`` times; counts identical to Orrery's for the same seed.

    ``precision`` ("c128" default, or "c64") and ``trajectory_mode`` ("serial" default: Orrery's
    draw order; "batched": all shots at once, each with its own uniforms) are optional engine
    knobs; defaults also come from ``LSG_PRECISION`` / ``LSG_TRAJ_MODE``. ``report_precision``
    (complex64 runs of static circuits; off by default, since it evolves the circuit again in
    complex128): ``Result.report["precision"]`` holds :func:`precision_report`'s errors."""
    if not 0 <= shots <= MAX_SHOTS:
        raise ValueError(f"shots must be between 0 and {MAX_SHOTS:,}")
    circuit = to_circuit(program, params)
    chosen = choose_method(circuit, noise, method)
    seed = secrets.randbelow(2**63) if seed is None else int(seed)
    if seed < 0:
        raise ValueError("seed must not be negative")
    if chosen in _ACCELERATORS:
        refuse_accelerator(chosen)
    rng = np.random.default_rng(seed)
    prec = engine.precision_code(precision)
    started = time.perf_counter()
    vector = None
    report: dict[str, Any] = {}
    if chosen == "stabilizer":
        from lucivant_sim_gb300 import stabilizer

        tally = stabilizer.run_counts(circuit, shots, noise, rng)
        counts = {format_bits(circuit, b): k for b, k in sorted(tally.items())} if circuit.num_clbits else {}
    elif chosen == "trajectories":
        from lucivant_sim_gb300 import trajectories

        if circuit.num_qubits > 0:
            engine.new_statevector(circuit.num_qubits, prec).free()  # size check before the shots
        tally, report = trajectories.run_shots(circuit, shots, noise, rng, prec, trajectory_mode)
        counts = {format_bits(circuit, b): k for b, k in sorted(tally.items())} if circuit.num_clbits else {}
    else:
        n = circuit.num_qubits
        if chosen == "statevector":
            reg = engine.new_statevector(n, prec)
            reg.apply_from_basis(engine.sv_oplist(circuit, fuse=True))
            dm = 0
        else:
            reg = engine.evolve_density(circuit, [noise], prec)
            dm = n
        with reg:
            if chosen == "statevector":
                vector = reg.download()[0]
            counts, report = sample_register(reg, circuit, dm, shots, noise, rng)
    elapsed = round(time.perf_counter() - started, 6)
    if report_precision and prec == _lib.C64 and chosen in ("statevector", "density_matrix"):
        report = dict(report, precision=precision_report(circuit, noise))
    return Result(
        counts=counts if chosen in ("statevector", "density_matrix") else dict(sorted(counts.items())),
        shots=shots,
        seed=seed,
        method=chosen,
        num_qubits=circuit.num_qubits,
        num_clbits=circuit.num_clbits,
        circuit_digest=circuit.digest(),
        noise_digest=noise.digest() if noise is not None and not noise.is_empty() else None,
        version=engine_version(),
        elapsed_seconds=elapsed,
        statevector=vector,
        report=report,
    )


def _static(circuit: Any, what: str) -> None:
    if circuit.is_dynamic():
        raise SimulationError(f"{what} needs a circuit without mid-circuit measurement or conditions")


def statevector(program: Any, params: Mapping[str, float] | None = None, *, precision: str | None = None) -> NDArray[np.complex128]:  # noqa: E501
    """The ideal final state (measurements ignored), little-endian."""
    circuit = to_circuit(program, params)
    _static(circuit, "a statevector")
    with engine.new_statevector(circuit.num_qubits, engine.precision_code(precision)) as reg:
        reg.apply_from_basis(engine.sv_oplist(circuit, fuse=True))
        return reg.download()[0]


def density_matrix(program: Any, noise: Any = None, params: Mapping[str, float] | None = None, *,
                   precision: str | None = None) -> NDArray[np.complex128]:  # fmt: skip
    """The final mixed state under ``noise`` (measurements ignored), shape (2^n, 2^n)."""
    circuit = to_circuit(program, params)
    _static(circuit, "a density matrix")
    n = circuit.num_qubits
    with engine.evolve_density(circuit, [noise], engine.precision_code(precision)) as reg:
        return engine.density_download(reg)


def probabilities_array(program: Any, noise: Any = None, params: Mapping[str, float] | None = None, *,
                        precision: str | None = None) -> NDArray[np.float64]:  # fmt: skip
    """Exact probabilities of every basis state, as an array (index bit q = qubit q)."""
    circuit = to_circuit(program, params)
    _static(circuit, "exact probabilities")
    reg, dm = _evolved(circuit, noise, engine.precision_code(precision))
    with reg:
        return reg.probabilities(dm)


def probabilities(program: Any, noise: Any = None, params: Mapping[str, float] | None = None, *,
                  threshold: float = 1e-12, precision: str | None = None) -> dict[str, float]:  # fmt: skip
    """Exact probabilities keyed by bitstring (qubit 0 rightmost), before readout error
    (``simulator.py:424-442``)."""
    circuit = to_circuit(program, params)
    probs = probabilities_array(circuit, noise, precision=precision)
    n = circuit.num_qubits
    keep = np.flatnonzero(probs > threshold)
    return {format(int(i), f"0{n}b"): float(probs[i]) for i in keep}


def outcome_probabilities(program: Any, noise: Any = None, params: Mapping[str, float] | None = None, *,
                          threshold: float = 1e-12, precision: str | None = None) -> dict[str, float]:  # fmt: skip
    """Exact outcome probabilities with readout error, keyed like ``Result.counts``
    (``simulator.py:445-486``)."""
    circuit = to_circuit(program, params)
    _static(circuit, "exact outcome probabilities")
    pairs = final_measurements(circuit)
    if not pairs:
        return {}
    reg, dm = _evolved(circuit, noise, engine.precision_code(precision))
    measured = sorted({q for q, _ in pairs})
    position = {q: i for i, q in enumerate(measured)}
    errs = []
    for q, _c in pairs:
        err = noise.readout_error(q) if noise else None
        errs.append((float(err.p01), float(err.p10)) if err is not None else (0.0, 0.0))
    with reg:  # the marginal, the threshold and every pair's readout flips run on the device
        space = reg.outcome_probabilities(dm, measured, [position[q] for q, _ in pairs], errs, threshold)
    out = deposit_pairs(space, [c for _, c in pairs], circuit.num_clbits)
    return {format_bits(circuit, b): w for b, w in sorted(out.items()) if w > threshold}


def deposit_pairs(space: NDArray[np.float64], clbits: list[int], num_clbits: int) -> dict[int, float]:
    """Outcome probabilities keyed by classical bits from the pair-bit space (index bit j = the
    bit pair j reported, written to classical bit ``clbits[j]``; pairs writing one classical bit
    combine by OR, as the reference packs them); nonzero entries only."""
    idx = np.flatnonzero(space)
    if num_clbits > 62:
        keys = [sum(((int(e) >> j) & 1) << c for j, c in enumerate(clbits)) for e in idx]
    else:
        packed = np.zeros(idx.size, dtype=np.int64)
        for j, c in enumerate(clbits):
            packed |= ((idx >> j) & 1).astype(np.int64) << c
        keys = packed.tolist()
    out: dict[int, float] = {}
    for k, w in zip(keys, space[idx].tolist(), strict=True):
        out[k] = out.get(k, 0.0) + w
    return out


def expectation(program: Any, observable: str | Mapping[str, float], noise: Any = None,
                params: Mapping[str, float] | None = None, *, precision: str | None = None) -> float:  # fmt: skip
    """<O> for a Pauli string (qubit 0 rightmost) or a weighted sum (``simulator.py:489-527``).
    All terms are evaluated on the device from one evolution."""
    circuit = to_circuit(program, params)
    _static(circuit, "an expectation value")
    terms = {observable: 1.0} if isinstance(observable, str) else dict(observable)
    n = circuit.num_qubits
    for label in terms:
        if len(label) != n or set(label.upper()) - set("IXYZ"):
            raise ValueError(f"{label!r} must be a Pauli string of length {n} (qubit 0 rightmost)")
    if not terms:
        return 0.0
    reg, dm = _evolved(circuit, noise, engine.precision_code(precision))
    masks = [pauli_masks(label) for label in terms]
    with reg:
        vals = reg.expect(dm, [m[0] for m in masks], [m[1] for m in masks])[:, 0]
    total = 0.0
    for w, v in zip(terms.values(), vals, strict=True):
        total += w * float(v)
    return total


def verify(saved: Mapping[str, Any] | str | Path, program: Any, noise: Any = None) -> bool:
    """Rerun a saved result and check the counts are identical (``simulator.py:539-547``)."""
    data = json.loads(Path(saved).read_text(encoding="utf-8")) if isinstance(saved, (str, Path)) else dict(saved)
    again = run(program, int(data["shots"]), seed=int(data["seed"]), noise=noise, method=str(data["method"]))
    if again.circuit_digest != data.get("circuit_digest"):
        return False
    if (again.noise_digest or None) != (data.get("noise_digest") or None):
        return False
    return again.counts_digest == data.get("counts_digest") and again.counts == data.get("counts")


__all__ = [
    "METHODS",
    "Circuit",
    "Result",
    "choose_method",
    "density_matrix",
    "expectation",
    "outcome_probabilities",
    "precision_report",
    "probabilities",
    "probabilities_array",
    "run",
    "statevector",
    "verify",
]
