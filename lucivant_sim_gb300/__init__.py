"""Orrery's simulation hot path on one GB300: the same API, hand-written sm_103a kernels.

    import lucivant_sim_gb300 as ls

    result = ls.run(qasm_source, shots=1000, seed=7)   # counts identical to Orrery's

Public functions and types mirror ``lucivant_sim`` 0.3.0 (``src/lucivant_sim/__init__.py:21-76``).
Beneath them a ctypes C ABI (``include/lsg.h``) drives the CUDA engine library ``liblsg.so``.
"""

from lucivant_sim_gb300._lib import EngineError, SimulationError
from lucivant_sim_gb300.circuit import Circuit
from lucivant_sim_gb300.clifford import is_clifford
from lucivant_sim_gb300.noise import (
    Channel,
    NoiseModel,
    ReadoutError,
    amplitude_damping,
    bit_flip,
    depolarizing,
    from_gate_error,
    pauli_channel,
    phase_damping,
    phase_flip,
    thermal_relaxation,
)
from lucivant_sim_gb300.qasm import QasmError, load, parse
from lucivant_sim_gb300.simulator import (
    METHODS,
    Result,
    __version__,
    choose_method,
    density_matrix,
    expectation,
    outcome_probabilities,
    precision_report,
    probabilities,
    probabilities_array,
    run,
    statevector,
    verify,
)

__all__ = [
    "METHODS",
    "Channel",
    "Circuit",
    "EngineError",
    "NoiseModel",
    "QasmError",
    "ReadoutError",
    "Result",
    "SimulationError",
    "__version__",
    "amplitude_damping",
    "bit_flip",
    "choose_method",
    "density_matrix",
    "depolarizing",
    "expectation",
    "from_gate_error",
    "is_clifford",
    "load",
    "outcome_probabilities",
    "precision_report",
    "parse",
    "pauli_channel",
    "phase_damping",
    "phase_flip",
    "probabilities",
    "probabilities_array",
    "run",
    "statevector",
    "thermal_relaxation",
    "verify",
]
