"""Batched execution: one circuit template, many instances, one register.

Noise-parameter instances (or shots, or repeated runs) of one circuit share every pass: the
register holds ``batch`` members contiguously and each operator carries per-member data where
the instances differ, so a pass over all members is one kernel launch. The template is planned
and uploaded once (:class:`~lucivant_sim_gb300._lib.Program`) and re-run without host
synchronisation.
"""

from __future__ import annotations

from typing import Any

import numpy as np

from lucivant_sim_gb300 import _lib, autotune as tuning, engine
from lucivant_sim_gb300.engine import pauli_masks


class DensityBatch:
    """``len(noises)`` noisy density-matrix instances of one static circuit.

    ``precision``: "c128" (FP64), "c64" (complex64 request: real32 in Pauli-transfer form) or
    "df64": the Pauli-transfer register in double-float pairs (two FP32 words per coefficient,
    FP32 arithmetic with exact error terms, about 48 significant bits); it needs the
    Pauli-transfer form (gates on at most two qubits)."""

    def __init__(self, circuit: Any, noises: list[Any], precision: str | None = "c64",
                 autotune: bool | None = None) -> None:  # fmt: skip
        if circuit.is_dynamic():
            raise engine.SimulationError("a density matrix needs a circuit without mid-circuit measurement or conditions")
        self.circuit = circuit
        self.n = circuit.num_qubits
        self.batch = len(noises)
        df64 = precision == "df64"
        prec = _lib.C128 if df64 else engine.precision_code(precision)
        self.form = engine.dm_form(circuit, noises)
        if df64 and self.form != "ptm":
            raise ValueError("double-float registers hold the Pauli-transfer form (gates on at most two qubits)")
        if self.form == "ptm":  # Pauli-transfer form: real coefficients, real channel matrices
            self.reg = engine.new_density(self.n, _lib.RD if df64 else engine.REAL_OF[prec], self.batch)
            self.ops = engine.ptm_oplist(circuit, noises)
        else:
            self.reg = engine.new_density(self.n, prec, self.batch)
            self.ops = engine.dm_oplist(circuit, noises)
        # plan choices searched on the device per program shape (autotune.py), when asked
        if tuning.wanted(autotune):
            self.program, self.tune = tuning.tuned_program(self.reg, self.ops)
        else:
            self.program, self.tune = _lib.Program(self.reg, self.ops), None
        self.upload_bytes = int(self.ops.size * 16 + len(self.ops) * _lib.OP_DTYPE.itemsize)

    @property
    def register_bytes(self) -> int:
        return _lib.ELEM_BYTES[self.reg.precision] * self.batch << (2 * self.n)

    def evolve(self) -> None:
        """Reset every member to |0><0| and run the circuit (queued; returns before completion).
        Tiles that the circuit has not reached yet are still zero and are skipped."""
        self.program.run_from_basis(self.reg, 0)

    def evolve_timed(self) -> np.ndarray:
        """As :meth:`evolve`, returning each fused pass's device time in ms."""
        return self.program.run_from_basis(self.reg, 0, timed=True)

    @property
    def bytes_per_evolve(self) -> int:
        """HBM bytes the passes of one :meth:`evolve` move."""
        return self.program.basis_bytes_per_run

    def probabilities(self) -> np.ndarray:
        """(batch, 2^n) exact probabilities."""
        return self.reg.probabilities(self.n, member=-1)

    def expectations(self, labels: list[str]) -> np.ndarray:
        """(terms, batch) Pauli expectations."""
        masks = [pauli_masks(lab) for lab in labels]
        return self.reg.expect(self.n, [m[0] for m in masks], [m[1] for m in masks])

    def free(self) -> None:
        self.program.free()
        self.reg.free()


def halves(noises: list[Any], split: bool = True) -> list[list[Any]]:
    """The batches :func:`run_density_batch` evolves: two equal halves of an even, non-empty
    batch with ``split``, else the whole batch."""
    if split and noises and len(noises) % 2 == 0:
        return [noises[: len(noises) // 2], noises[len(noises) // 2 :]]
    return [noises]


def run_density_batch(
    circuit: Any, noises: list[Any], observables: list[str], precision: str | None = "c64", split: bool = True,
    autotune: bool | None = None,
):
    """One call from host inputs to host results: probabilities (batch, 2^n) and expectations
    (terms, batch) of every noise instance.

    With ``split`` an even batch runs as two halves of one shape: the second half's operators are
    built on the host while the first half evolves on the device, so most host work hides behind
    device work. Every member's result is the same as in one whole batch (members evolve
    independently). A half that the library would not specialize while the whole batch would be
    (a run of the whole moves twice the bytes) is dropped for the whole batch."""
    parts = halves(noises, split)
    done: list[DensityBatch] = []
    try:
        first = DensityBatch(circuit, parts[0], precision, autotune)
        done.append(first)
        if len(parts) == 2 and not first.program.specialized:
            nominal = first.program.bytes_per_run
            if not _lib.jit_wanted(nominal) and _lib.jit_wanted(2 * nominal):
                done.pop().free()  # the whole batch would be specialized: run it as one
                parts = [noises]
                first = DensityBatch(circuit, noises, precision, autotune)
                done.append(first)
        first.evolve()
        for part in parts[1:]:
            b = DensityBatch(circuit, part, precision, autotune)
            done.append(b)
            b.evolve()
        probs = [b.probabilities() for b in done]
        exps = [b.expectations(observables) for b in done]
        if len(done) == 1:
            return probs[0], exps[0]
        return np.concatenate(probs, axis=0), np.concatenate(exps, axis=1)
    finally:
        for b in done:
            b.free()
