"""Record Orrery's noise models (lucivant-sim 0.3.0, ``noise.py``) by running Orrery itself: every
channel factory over several parameters (Kraus operators, mixture branches, description), the
factories' refusals, the rule each (gate, qubits) query resolves to in models with overlapping
rules, readout lookups, descriptions and digests, and models read from calibrations.

Run from the repository root, in a checkout where Orrery's sources are readable:

    python tests/golden/make_golden_noise.py /path/to/lucivant-sim/src

It writes ``tests/golden/noise.json`` and ``tests/golden/noise.npz``. The recipes are data
(``CHANNELS``, ``MODELS``, ``CALIBRATIONS``) applied to either module by ``recipes.build_channel``
and ``recipes.build_model``, so the tests build the same objects with the engine's module.
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

sys.dont_write_bytecode = True
HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

from recipes import build_channel, build_model  # noqa: E402

# (factory, args) — each is called as getattr(module, factory)(*args)
CHANNELS = [
    ("depolarizing", [0.0]), ("depolarizing", [0.01]), ("depolarizing", [0.75]), ("depolarizing", [4 / 3]),
    ("depolarizing", [0.02, 2]), ("depolarizing", [16 / 15, 2]), ("depolarizing", [0.1, 3]),
    ("from_gate_error", [0.001, 1]), ("from_gate_error", [0.01, 2]), ("from_gate_error", [0.9, 1]),
    ("bit_flip", [0.0]), ("bit_flip", [0.3]), ("phase_flip", [0.25]), ("phase_flip", [1.0]),
    ("amplitude_damping", [0.0]), ("amplitude_damping", [0.1]), ("amplitude_damping", [1.0]),
    ("phase_damping", [0.2]), ("phase_damping", [1.0]),
    ("thermal_relaxation", [120, 90, 0.05]), ("thermal_relaxation", [50, 40, 3.0]),
    ("thermal_relaxation", [20, 15, 4.0]), ("thermal_relaxation", [10, 20, 1.0]), ("thermal_relaxation", [30, 30, 0.0]),
    ("pauli_channel", [{"X": 0.1, "Z": 0.05}]), ("pauli_channel", [{"XY": 0.03, "ZZ": 0.02, "IX": 0.01}]),
    ("pauli_channel", [{"Y": 0.5, "X": 0.5}]), ("pauli_channel", [{"I": 0.2, "Z": 0.0}]),
]  # fmt: skip

BAD_CHANNELS = [
    ("depolarizing", [-0.1]), ("depolarizing", [1.5]), ("depolarizing", [float("nan")]), ("bit_flip", [1.2]),
    ("phase_flip", [-1e-9]), ("amplitude_damping", [2.0]), ("phase_damping", [-0.5]),
    ("thermal_relaxation", [10, 30, 1.0]), ("thermal_relaxation", [0, 0, 1.0]), ("thermal_relaxation", [10, 5, -1.0]),
    ("pauli_channel", [{"X": 0.7, "Z": 0.6}]), ("pauli_channel", [{"XA": 0.1}]), ("pauli_channel", [{"X": 0.1, "YZ": 0.1}]),
]  # fmt: skip

# a model is a list of steps: ["gate", channel recipe, gates, qubits] or ["readout", value, qubits]
# (value a float or [p01, p10]) or ["uniform", single, two, readout]
MODELS = {
    "empty": [],
    "uniform": [["uniform", 1e-3, 1e-2, 2e-2]],
    "uniform_no_readout": [["uniform", 1e-3, 0.0, 0.0]],
    "specificity": [
        ["gate", ["depolarizing", [0.01]], None, None],
        ["gate", ["bit_flip", [0.02]], "x", None],
        ["gate", ["phase_flip", [0.03]], None, [2]],
        ["gate", ["amplitude_damping", [0.04]], ["h", "x"], [2]],
        ["gate", ["depolarizing", [0.05, 2]], None, None],
        ["gate", ["depolarizing", [0.06, 2]], "cx", [1, 0]],
        ["gate", ["phase_damping", [0.07]], "rz", None],
        ["gate", ["depolarizing", [0.08]], None, None],
        ["readout", 0.01, None], ["readout", [0.02, 0.05], [1, 3]],
    ],
    "aliases": [
        ["gate", ["bit_flip", [0.1]], ["cnot", "u"], None],
        ["gate", ["depolarizing", [0.02, 2]], "CX", None],
        ["gate", ["phase_flip", [0.2]], "U", [0]],
    ],
    "thermal_over_uniform": [["uniform", 1e-3, 1e-2, 2e-2], ["gate", ["thermal_relaxation", [120, 90, 0.05]], "u3", None]],
    "readout_only": [["readout", [0.0, 0.0], None], ["readout", 0.03, [2]]],
}

QUERIES = [
    ["x", [0]], ["x", [2]], ["h", [2]], ["h", [0]], ["y", [2]], ["rz", [0]], ["rz", [2]], ["p", [1]], ["u1", [1]],
    ["id", [0]], ["u3", [1]], ["u", [0]], ["cx", [0, 1]], ["cx", [1, 0]], ["cx", [2, 3]], ["cnot", [0, 1]],
    ["cz", [1, 0]], ["swap", [3, 1]], ["ccx", [0, 1, 2]], ["sx", [3]], ["U", [0]], ["CX", [0, 1]], ["gphase", []],
]  # fmt: skip

CALIBRATIONS = [
    {"device": "twin-a", "single_qubit_error": 0.001, "two_qubit_error": 0.01, "readout_error": 0.02},
    {"profile_key": "p1", "single_qubit_error": None, "two_qubit_error": 0.02,
     "qubits": [{"qubit": 0, "single_qubit_error": 0.003, "readout_error": 0.04}, {"qubit": 2, "readout_error": None}],
     "couplers": [{"qubits": [0, 1], "error": 0.015}, {"qubits": [1, 2], "error": None}]},
    {"calibration": {"device": "wrapped", "readout_error": 0.05, "qubits": [{"qubit": 1, "single_qubit_error": 0.002}]}},
    {},
]  # fmt: skip


def channel_record(ch, arrays: dict, key: str) -> dict:
    arrays[f"{key}::kraus"] = np.stack([np.asarray(k, dtype=np.complex128) for k in ch.kraus])
    rec = {"name": ch.name, "num_qubits": ch.num_qubits, "describe": ch.describe(), "kraus": len(ch.kraus),
           "mixture": None if ch.mixture is None else [float(p) for p, _m in ch.mixture],
           "analytic_depolarizing": bool(getattr(ch, "analytic_depolarizing", False))}  # fmt: skip
    if ch.mixture is not None:
        arrays[f"{key}::mixture"] = np.stack([np.asarray(m, dtype=np.complex128) for _p, m in ch.mixture])
    return rec


def main(ref_src: str) -> None:
    sys.path.insert(0, ref_src)
    import lucivant_sim as ls
    from lucivant_sim import noise as ns

    arrays: dict[str, np.ndarray] = {}
    out: dict[str, object] = {"reference_version": ls.__version__, "channels": [], "bad_channels": [], "models": {},
                              "calibrations": []}  # fmt: skip
    for i, recipe in enumerate(CHANNELS):
        out["channels"].append({"recipe": recipe, **channel_record(build_channel(ns, recipe), arrays, f"ch{i}")})
    for recipe in BAD_CHANNELS:
        try:
            build_channel(ns, recipe)
            rec = {"recipe": recipe, "error": None}
        except Exception as exc:  # noqa: BLE001 - the class and message are the record
            rec = {"recipe": recipe, "error": {"class": type(exc).__name__, "message": str(exc)}}
        out["bad_channels"].append(rec)
    for name, steps in MODELS.items():
        m = build_model(ns, steps)
        answers = []
        for gate, qubits in QUERIES:
            ch = m.gate_error(gate, tuple(qubits))
            answers.append(None if ch is None else ch.describe())
        readout = []
        for q in range(5):
            e = m.readout_error(q)
            readout.append(None if e is None else [e.p01, e.p10])
        out["models"][name] = {"steps": steps, "describe": m.describe(), "digest": m.digest(),
                               "has_gate_errors": m.has_gate_errors(), "is_empty": m.is_empty(),
                               "source": m.source, "gate_error": answers, "readout_error": readout}  # fmt: skip
    try:
        build_model(ns, [["gate", ["depolarizing", [0.1, 2]], None, [0]]])
        bad_attach = None
    except Exception as exc:  # noqa: BLE001
        bad_attach = {"class": type(exc).__name__, "message": str(exc)}
    out["bad_attach"] = bad_attach
    for cal in CALIBRATIONS:
        m = ns.NoiseModel.from_calibration(cal)
        out["calibrations"].append({"calibration": cal, "describe": m.describe(), "digest": m.digest(), "source": m.source})
    out["queries"] = QUERIES
    np.savez_compressed(HERE / "noise.npz", **arrays)
    (HERE / "noise.json").write_text(json.dumps(out, indent=1, sort_keys=True))
    print("wrote", HERE / "noise.json", HERE / "noise.npz")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden_noise.py /path/to/lucivant-sim/src")
    main(sys.argv[1])
