"""Record Orrery's method choice (lucivant-sim 0.3.0, ``simulator.choose_method``) for every method
name over circuits and noise models that exercise each of its rules, by running Orrery itself.

Run from the repository root, in a checkout where Orrery's sources are readable:

    python tests/golden/make_golden_methods.py /path/to/lucivant-sim/src

It writes ``tests/golden/methods.json``: per case the OpenQASM text, the noise model's name (built
the same way on both sides by ``recipes.noise_model``), the requested method and Orrery's answer (the
chosen method, or the exception's class name and message). The tests never need Orrery.
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

sys.dont_write_bytecode = True
HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

from recipes import noise_model  # noqa: E402

METHODS = ("automatic", "statevector", "density_matrix", "trajectories", "stabilizer", "statevector_aer",
           "stabilizer_stim", "no_such_method")  # fmt: skip


def _program(n: int, body: str, bits: int = 0) -> str:
    head = ["OPENQASM 3.0;", 'include "stdgates.inc";', f"qubit[{n}] q;"]
    if bits:
        head.append(f"bit[{bits}] c;")
    return "\n".join(head) + "\n" + body + "\n"


def _chain(n: int, gate: str = "h") -> str:
    return " ".join(f"{gate} q[{i}];" for i in range(n)) + " " + " ".join(f"cx q[{i}], q[{i + 1}];" for i in range(n - 1))


PROGRAMS = {
    "clifford4": _program(4, _chain(4) + " c = measure q;", 4),
    "clifford11": _program(11, _chain(11) + " c = measure q;", 11),
    "clifford12": _program(12, _chain(12) + " c = measure q;", 12),
    "clifford12_t": _program(12, _chain(12) + " t q[5]; c = measure q;", 12),
    "clifford12_dynamic": _program(12, _chain(12) + " c[0] = measure q[0]; if (c[0] == 1) x q[3]; c = measure q;", 12),
    "clifford12_reset": _program(12, _chain(12) + " reset q[2]; c = measure q;", 12),
    "u3_6": _program(6, " ".join(f"u3(0.{i + 1}, 0.2, 0.3) q[{i}];" for i in range(6)) + " cx q[0], q[1]; c = measure q;", 6),
    "u3_10": _program(10, " ".join(f"ry(0.{i + 1}) q[{i}];" for i in range(10)) + " cx q[0], q[9]; c = measure q;", 10),
    "u3_11": _program(11, " ".join(f"ry(0.{i + 1}) q[{i}];" for i in range(11)) + " cx q[0], q[10]; c = measure q;", 11),
    "u3_14": _program(14, " ".join(f"rx(0.{i % 9 + 1}) q[{i}];" for i in range(14)) + " c = measure q;", 14),
    "dynamic_u3_6": _program(6, "ry(0.4) q[0]; c[0] = measure q[0]; if (c[0] == 1) x q[1]; c = measure q;", 6),
    "wide_clifford_3q": _program(12, _chain(12) + " ccx q[0], q[1], q[2]; c = measure q;", 12),
}

NOISES = ("none", "empty", "pauli", "readout_only", "damping_on_h", "depolarizing_on_cx")


def main(ref_src: str) -> None:
    sys.path.insert(0, ref_src)
    import lucivant_sim as ls
    from lucivant_sim import noise as ns
    from lucivant_sim.simulator import choose_method

    cases = []
    for pname, src in PROGRAMS.items():
        circuit = ls.parse(src)
        for nname in NOISES:
            nm = noise_model(nname, ns)
            for method in METHODS:
                try:
                    answer = {"method": choose_method(circuit, nm, method)}
                except Exception as exc:  # noqa: BLE001 - the class and message are the record
                    answer = {"error": type(exc).__name__, "message": str(exc)}
                cases.append({"program": pname, "noise": nname, "method": method, **answer})
    out = {"reference_version": ls.__version__, "programs": PROGRAMS, "cases": cases}
    (HERE / "methods.json").write_text(json.dumps(out, indent=1, sort_keys=True))
    print("wrote", HERE / "methods.json", len(cases), "cases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden_methods.py /path/to/lucivant-sim/src")
    main(sys.argv[1])
