"""How the golden fixtures' noise models are built, as data applied to a noise module.

The fixture generators build Orrery's objects with these functions and the tests build the
engine's with the same calls, so both sides hold the same models. Imported by both; no side
effects.
"""

from __future__ import annotations

from typing import Any


def build_channel(ns: Any, recipe: list) -> Any:
    """``recipe`` = [factory name, arguments]: ``getattr(ns, factory)(*arguments)``."""
    name, args = recipe
    return getattr(ns, name)(*args)


def build_model(ns: Any, steps: list) -> Any:
    """A NoiseModel from steps: ["gate", channel recipe, gates, qubits], ["readout", value,
    qubits] (value a float or [p01, p10]) or ["uniform", single, two, readout]."""
    model = ns.NoiseModel()
    for step in steps:
        if step[0] == "uniform":
            fresh = ns.NoiseModel.uniform(single=step[1], two=step[2], readout=step[3])
            model.rules.extend(fresh.rules)
            model.readout.update(fresh.readout)
            model.source = fresh.source
        elif step[0] == "gate":
            model.add_gate_error(build_channel(ns, step[1]), gates=step[2], qubits=step[3])
        else:
            value = step[1]
            err = ns.ReadoutError(*value) if isinstance(value, list) else value
            model.add_readout_error(err, qubits=step[2])
    return model


def noise_model(name: str, ns: Any) -> Any:
    """The method-choice fixture's named noise models."""
    if name == "none":
        return None
    if name == "empty":
        return ns.NoiseModel()
    if name == "pauli":
        return ns.NoiseModel.uniform(single=1e-3, two=1e-2, readout=2e-2)
    if name == "readout_only":
        return ns.NoiseModel.uniform(readout=3e-2)
    if name == "damping_on_h":
        return ns.NoiseModel().add_gate_error(ns.amplitude_damping(0.1), gates="h")
    if name == "depolarizing_on_cx":
        return ns.NoiseModel().add_gate_error(ns.depolarizing(0.02, 2), gates="cx")
    raise KeyError(name)
