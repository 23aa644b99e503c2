"""Record Orrery's simulation results through its public functions (lucivant-sim 0.3.0: ``run``,
``probabilities``, ``outcome_probabilities``, ``expectation``, ``statevector``, ``density_matrix``)
on seeded random programs with varied measurement layouts, by running Orrery itself.

Run from the repository root, in a checkout where Orrery's sources are readable:

    python tests/golden/make_golden_sim.py /path/to/lucivant-sim/src

It writes ``tests/golden/sim.json`` and ``tests/golden/sim.npz``. Each case is OpenQASM text, a
noise recipe (``tests/golden/make_golden_noise.py``'s model steps), a seed and Orrery's results;
the tests never need Orrery.

The programs draw gates from every one- and two-qubit gate name, several three-qubit ones and
modifiers, and measure into two classical registers in layouts Orrery allows: a qubit measured
into two bits, a bit written twice (the later measurement wins), bits left unmeasured. Run-only
cases add programs with mid-circuit measurement, conditions and reset (Orrery's trajectories) and
random Clifford layers over every Clifford gate name at 12 to 16 qubits (its stabilizer engine).
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

sys.dont_write_bytecode = True
HERE = Path(__file__).resolve().parent

ONE = ["h", "x", "y", "z", "s", "sdg", "t", "tdg", "sx", "sxdg", "id"]
ONE_P = [("rx", 1), ("ry", 1), ("rz", 1), ("p", 1), ("u2", 2), ("u3", 3), ("u", 3)]
TWO = ["cx", "cy", "cz", "ch", "csx", "swap", "iswap", "ecr", "dcx"]
TWO_P = [("cp", 1), ("crx", 1), ("cry", 1), ("crz", 1), ("rxx", 1), ("ryy", 1), ("rzz", 1), ("rzx", 1), ("cu3", 3),
         ("cu", 4)]  # fmt: skip
THREE = ["ccx", "ccz", "cswap"]
MODIFIED = ["ctrl @ h", "negctrl @ x", "inv @ t", "pow(0.5) @ x", "inv @ pow(2) @ sx"]

NOISES = {
    "none": None,
    "uniform": [["uniform", 2e-3, 1.5e-2, 3e-2]],
    "mixed": [["gate", ["amplitude_damping", [0.05]], "h", None], ["gate", ["phase_damping", [0.1]], None, [1]],
              ["gate", ["depolarizing", [0.03, 2]], None, None], ["gate", ["thermal_relaxation", [40, 30, 2.0]], "u3", None],
              ["readout", [0.02, 0.06], None], ["readout", 0.1, [0]]],  # fmt: skip
    "readout_only": [["readout", [0.03, 0.08], None]],
}


def program(n: int, depth: int, seed: int, layout: str) -> str:
    rng = np.random.default_rng(seed)
    lines = ["OPENQASM 3.0;", 'include "stdgates.inc";', f"qubit[{n}] q;", "bit[3] c;", "bit[2] d;"]
    for _ in range(depth):
        kind = rng.integers(6)
        qs = [int(v) for v in rng.permutation(n)]
        if kind == 0:
            lines.append(f"{ONE[rng.integers(len(ONE))]} q[{qs[0]}];")
        elif kind == 1:
            name, k = ONE_P[rng.integers(len(ONE_P))]
            ps = ", ".join(repr(float(v)) for v in rng.uniform(-3.2, 3.2, size=k))
            lines.append(f"{name}({ps}) q[{qs[0]}];")
        elif kind == 2:
            lines.append(f"{TWO[rng.integers(len(TWO))]} q[{qs[0]}], q[{qs[1]}];")
        elif kind == 3:
            name, k = TWO_P[rng.integers(len(TWO_P))]
            ps = ", ".join(repr(float(v)) for v in rng.uniform(-3.2, 3.2, size=k))
            lines.append(f"{name}({ps}) q[{qs[0]}], q[{qs[1]}];")
        elif kind == 4 and n >= 3:
            lines.append(f"{THREE[rng.integers(len(THREE))]} q[{qs[0]}], q[{qs[1]}], q[{qs[2]}];")
        else:
            mod = MODIFIED[rng.integers(len(MODIFIED))]
            operands = f"q[{qs[0]}], q[{qs[1]}]" if mod.startswith(("ctrl", "negctrl")) else f"q[{qs[0]}]"
            lines.append(f"{mod} {operands};")
    if layout == "all":
        lines.append(f"bit[{n}] m;")
        lines.append("m = measure q;")
    elif layout == "split":  # q[0] into c[0] and d[1]; c[1] unmeasured; c[2] written twice
        lines += ["c[0] = measure q[0];", "d[1] = measure q[0];", f"c[2] = measure q[{n - 1}];",
                  f"d[0] = measure q[{n - 2}];", f"c[2] = measure q[1];"]  # fmt: skip
    else:  # none measured
        pass
    return "\n".join(lines) + "\n"


CASES = [
    # (name, qubits, depth, program seed, layout, noise, run seed)
    ("sv5_all", 5, 30, 1, "all", "none", 11),
    ("sv6_split", 6, 40, 2, "split", "none", 12),
    ("sv7_all_readout", 7, 45, 3, "all", "readout_only", 13),
    ("sv4_split_readout", 4, 25, 4, "split", "readout_only", 14),
    ("sv6_nomeasure", 6, 30, 5, "none", "none", 15),
    ("dm4_all_uniform", 4, 25, 6, "all", "uniform", 16),
    ("dm5_split_uniform", 5, 30, 7, "split", "uniform", 17),
    ("dm4_split_mixed", 4, 20, 8, "split", "mixed", 18),
    ("dm5_all_mixed", 5, 25, 9, "all", "mixed", 19),
    ("dm3_all_mixed", 3, 15, 10, "all", "mixed", 20),
]

CLIFFORD_ONE = ["h", "s", "sdg", "x", "y", "z", "sx", "sxdg", "id"]
CLIFFORD_TWO = ["cx", "cy", "cz", "swap", "iswap", "ecr", "dcx"]


def dynamic_program(n: int, rounds: int, seed: int) -> str:
    """Rounds of random one- and two-qubit gates, a mid-circuit measurement, a condition on it
    (a gate, or an if/else block) and a reset; all qubits measured at the end."""
    rng = np.random.default_rng(seed)
    lines = ["OPENQASM 3.0;", 'include "stdgates.inc";', f"qubit[{n}] q;", f"bit[{n}] c;", "bit[2] m;"]
    for r in range(rounds):
        for q in range(n):
            ps = ", ".join(repr(float(v)) for v in rng.uniform(-3.2, 3.2, size=3))
            lines.append(f"u3({ps}) q[{q}];")
        a = int(rng.integers(n - 1))
        lines.append(f"cx q[{a}], q[{a + 1}];")
        mq = int(rng.integers(n))
        lines.append(f"m[{r % 2}] = measure q[{mq}];")
        t = (mq + 1) % n
        if r % 2:
            lines.append(f"if (m[{r % 2}] == 1) {{ x q[{t}]; h q[{(t + 1) % n}]; }} else {{ ry(0.7) q[{t}]; }}")
        else:
            lines.append(f"if (m == {int(rng.integers(4))}) z q[{t}];")
        lines.append(f"reset q[{int(rng.integers(n))}];")
    lines.append("c = measure q;")
    return "\n".join(lines) + "\n"


def clifford_program(n: int, layers: int, seed: int) -> str:
    """Random Clifford layers on ``n`` qubits (every Clifford gate name), measured into one register
    in a permuted order, a few qubits left unmeasured."""
    rng = np.random.default_rng(seed)
    lines = ["OPENQASM 3.0;", 'include "stdgates.inc";', f"qubit[{n}] q;", f"bit[{n - 2}] c;"]
    for _ in range(layers):
        for q in range(n):
            lines.append(f"{CLIFFORD_ONE[rng.integers(len(CLIFFORD_ONE))]} q[{q}];")
        order = [int(v) for v in rng.permutation(n)]
        for i in range(0, n - 1, 2):
            lines.append(f"{CLIFFORD_TWO[rng.integers(len(CLIFFORD_TWO))]} q[{order[i]}], q[{order[i + 1]}];")
    for i, q in enumerate(int(v) for v in rng.permutation(n)[: n - 2]):
        lines.append(f"c[{i}] = measure q[{q}];")
    return "\n".join(lines) + "\n"


# run-only cases (Orrery's expectations and probabilities refuse dynamic circuits):
# (name, program kind, qubits, size, program seed, noise, run seed, shots)
RUN_CASES = [
    ("traj5_ideal", "dynamic", 5, 3, 31, "none", 41, 400),
    ("traj6_uniform", "dynamic", 6, 3, 32, "uniform", 42, 300),
    ("traj4_mixed", "dynamic", 4, 4, 33, "mixed", 43, 300),
    ("stab14_ideal", "clifford", 14, 6, 34, "none", 44, 500),
    ("stab16_uniform", "clifford", 16, 5, 35, "uniform", 45, 500),
    ("stab12_readout", "clifford", 12, 8, 36, "readout_only", 46, 500),
]

OBSERVABLES = [lambda n: "Z" * n, lambda n: {"X" + "I" * (n - 1): 0.5, "I" * (n - 2) + "YZ": -1.25, "Z" * n: 0.75}]


def main(ref_src: str) -> None:
    sys.path.insert(0, ref_src)
    sys.path.insert(0, str(HERE))
    import lucivant_sim as ls
    from lucivant_sim import noise as ns
    from recipes import build_model

    arrays: dict[str, np.ndarray] = {}
    cases = []
    for name, n, depth, pseed, layout, noise_name, seed in CASES:
        src = program(n, depth, pseed, layout)
        steps = NOISES[noise_name]
        nm = None if steps is None else build_model(ns, steps)
        rec: dict[str, object] = {"name": name, "qasm": src, "noise": noise_name, "seed": seed}
        r = ls.run(src, shots=3000, seed=seed, noise=nm)
        rec.update(method=r.method, counts=r.counts, fingerprint_noise=r.noise_digest, circuit_digest=r.circuit_digest)
        rec["probabilities"] = ls.probabilities(src, nm)
        rec["outcome_probabilities"] = ls.outcome_probabilities(src, nm) if layout != "none" else {}
        rec["expectations"] = [ls.expectation(src, obs(n), nm) for obs in OBSERVABLES]
        rec["observables"] = [obs(n) for obs in OBSERVABLES]
        if nm is None or not nm.has_gate_errors():
            arrays[f"{name}::statevector"] = ls.statevector(src)
        else:
            arrays[f"{name}::density_matrix"] = ls.density_matrix(src, nm)
        cases.append(rec)
    run_cases = []
    for name, kind, n, size, pseed, noise_name, seed, shots in RUN_CASES:
        src = dynamic_program(n, size, pseed) if kind == "dynamic" else clifford_program(n, size, pseed)
        steps = NOISES[noise_name]
        nm = None if steps is None else build_model(ns, steps)
        r = ls.run(src, shots=shots, seed=seed, noise=nm)
        run_cases.append({"name": name, "qasm": src, "noise": noise_name, "seed": seed, "shots": shots,
                          "method": r.method, "counts": r.counts, "circuit_digest": r.circuit_digest,
                          "fingerprint_noise": r.noise_digest, "fingerprint": r.fingerprint})  # fmt: skip
    np.savez_compressed(HERE / "sim.npz", **arrays)
    (HERE / "sim.json").write_text(json.dumps({"reference_version": ls.__version__, "noises": NOISES, "cases": cases,
                                               "run_cases": run_cases}, indent=1, sort_keys=True))  # fmt: skip
    print("wrote", HERE / "sim.json", HERE / "sim.npz", len(cases), "cases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden_sim.py /path/to/lucivant-sim/src")
    main(sys.argv[1])
