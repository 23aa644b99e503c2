"""Generate the golden fixtures by running Orrery (lucivant-sim 0.3.0) itself.

Run from the repository root, in a checkout where Orrery's sources are readable:

    python tests/golden/make_golden.py /path/to/lucivant-sim/src

It writes ``tests/golden/golden.npz`` (statevectors, density matrices, probabilities, tableaux)
and ``tests/golden/golden.json`` (counts, expectations, outcome probabilities, digests). The
programs are the package's own seeded workloads at small sizes; their QASM text is stored too,
so the tests never need Orrery at run time.
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

sys.dont_write_bytecode = True
HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from lucivant_sim_gb300 import workloads as wl  # noqa: E402
from lucivant_sim_gb300.gates import GATES  # noqa: E402


def all_gates_program(seed: int) -> str:
    rng = np.random.default_rng(seed)
    lines = ["OPENQASM 3.0;", 'include "stdgates.inc";', "qubit[5] q;"]
    for q in range(5):
        lines.append(f"u3({float(rng.uniform(0, 6.28))!r}, {float(rng.uniform(0, 6.28))!r}, 0.3) q[{q}];")
    for name, spec in sorted(GATES.items()):
        qs = rng.permutation(5)[: spec.qubits]
        ps = ", ".join(repr(float(v)) for v in rng.uniform(-3, 3, size=spec.params))
        head = f"{name}({ps})" if spec.params else name
        lines.append(f"{head} " + ", ".join(f"q[{int(q)}]" for q in qs) + ";")
    lines.append("rccx q[0], q[2], q[4];")
    lines.append("rc3x q[4], q[3], q[1], q[0];")
    lines.append("ctrl @ u3(0.4, 0.5, 0.6) q[1], q[3];")
    lines.append("inv @ pow(0.5) @ sx q[2];")
    return "\n".join(lines) + "\n"


CHANNELS = """OPENQASM 3.0;
include "stdgates.inc";
qubit[4] q;
bit[4] c;
reset q[3]; h q[0]; cx q[0], q[1]; ry(0.7) q[2]; t q[1]; sx q[2]; cz q[1], q[2]; h q[2]; ry(1.3) q[3];
cx q[3], q[0];
c = measure q;
"""

DYNAMIC_CLIFFORD = """OPENQASM 3.0;
include "stdgates.inc";
qubit[14] q;
bit[14] c;
h q[0]; cx q[0], q[1]; h q[2]; s q[2]; cx q[2], q[3]; h q[5]; cz q[5], q[6]; h q[6];
c[0] = measure q[0];
if (c[0] == 1) x q[4];
reset q[1];
h q[1]; cx q[1], q[7];
c[2] = measure q[2];
if (c[2] == 0) { h q[8]; cx q[8], q[9]; }
h q[10]; sdg q[10]; cx q[10], q[11]; swap q[11], q[12]; cy q[12], q[13];
c = measure q;
"""

PARTIAL_CLIFFORD = """OPENQASM 3.0;
include "stdgates.inc";
qubit[20] q;
bit[7] c;
h q[0]; h q[3]; cx q[0], q[5]; cx q[3], q[9]; h q[11]; s q[11]; cx q[11], q[12]; cx q[5], q[12];
h q[15]; cz q[15], q[16]; h q[16]; cx q[9], q[19]; sx q[7]; swap q[7], q[2];
c[0] = measure q[12]; c[1] = measure q[0]; c[2] = measure q[9]; c[3] = measure q[16];
c[4] = measure q[19]; c[5] = measure q[2]; c[6] = measure q[5];
"""


def main(ref_src: str) -> None:
    sys.path.insert(0, ref_src)
    import lucivant_sim as ls
    from lucivant_sim import stabilizer as stab

    arrays: dict[str, np.ndarray] = {}
    meta: dict[str, object] = {"reference_version": ls.__version__, "cases": {}}
    cases = meta["cases"]

    def put(name: str, **info: object) -> None:
        cases[name] = info

    # statevector brickwork, config-1 shape at 8 qubits
    src = wl.brickwork(8, 6, seed=7)
    arrays["sv_bw8_state"] = ls.statevector(src)
    r = ls.run(src, shots=3000, seed=7)
    put("sv_bw8", qasm=src, shots=3000, seed=7, counts=r.counts, method=r.method,
        circuit_digest=r.circuit_digest, fingerprint=r.fingerprint, counts_digest=r.counts_digest)
    # readout error on a statevector run
    noise_ro = ls.NoiseModel().add_readout_error(ls.ReadoutError(0.05, 0.1))
    r = ls.run(src, shots=2000, seed=13, noise=noise_ro)
    put("sv_bw8_readout", qasm=src, shots=2000, seed=13, counts=r.counts, method=r.method)

    # every built-in gate
    src = all_gates_program(5)
    arrays["sv_gates_state"] = ls.statevector(src)
    put("sv_gates", qasm=src)

    # density matrix, config-2 shape at 4 qubits
    src = wl.brickwork(4, 3, seed=3)
    noise = ls.NoiseModel.uniform(single=1e-3, two=1e-2, readout=2e-2).add_gate_error(
        ls.thermal_relaxation(t1=120, t2=90, time=0.05), gates="u3"
    )
    arrays["dm_bw4_rho"] = ls.density_matrix(src, noise)
    r = ls.run(src, shots=4000, seed=5, noise=noise)
    zs = {}
    for i in range(4):
        lab = ["I"] * 4
        lab[3 - i] = "Z"
        zs["".join(lab)] = ls.expectation(src, "".join(lab), noise)
    for i in range(3):
        lab = ["I"] * 4
        lab[3 - i] = "Z"
        lab[3 - i - 1] = "Z"
        zs["".join(lab)] = ls.expectation(src, "".join(lab), noise)
    put("dm_bw4", qasm=src, shots=4000, seed=5, counts=r.counts, method=r.method, expectations=zs,
        outcome_probabilities=ls.outcome_probabilities(src, noise), noise_digest=r.noise_digest)

    # every channel kind on a small density matrix
    nz = (
        ls.NoiseModel()
        .add_gate_error(ls.amplitude_damping(0.1), gates="h")
        .add_gate_error(ls.phase_damping(0.2), gates="ry")
        .add_gate_error(ls.bit_flip(0.05), gates="t")
        .add_gate_error(ls.phase_flip(0.07), gates="sx")
        .add_gate_error(ls.pauli_channel({"XY": 0.03, "ZZ": 0.02, "IX": 0.01}), gates="cx")
        .add_gate_error(ls.depolarizing(0.2, 2), gates="cz")
        .add_gate_error(ls.thermal_relaxation(50, 40, 3.0), qubits=[2])
        .add_readout_error(ls.ReadoutError(0.02, 0.04), qubits=[0])
    )
    arrays["dm_channels_rho"] = ls.density_matrix(CHANNELS, nz)
    put("dm_channels", qasm=CHANNELS, outcome_probabilities=ls.outcome_probabilities(CHANNELS, nz))

    # trajectories with mid-circuit measurement, config-3 shape at 8 qubits
    src = wl.midcircuit(8, 2, seed=3)
    nz3 = ls.NoiseModel.uniform(single=2e-2, two=5e-2, readout=3e-2)
    r = ls.run(src, shots=300, seed=9, noise=nz3)
    put("traj_mid8", qasm=src, shots=300, seed=9, counts=r.counts, method=r.method)
    r = ls.run(src, shots=200, seed=4)
    put("traj_mid8_ideal", qasm=src, shots=200, seed=4, counts=r.counts, method=r.method)
    nzk = ls.NoiseModel().add_gate_error(ls.thermal_relaxation(20, 15, 4.0), gates="u3")
    r = ls.run(CHANNELS, shots=400, seed=21, noise=nzk, method="trajectories")
    put("traj_kraus", qasm=CHANNELS, shots=400, seed=21, counts=r.counts, method=r.method)

    # stabilizer: noisy frames, config-4 shape at 64 qubits
    src = wl.clifford_layers(64, 8, seed=11)
    nzs = ls.NoiseModel()
    nzs.add_gate_error(ls.depolarizing(1e-2, 1)).add_gate_error(ls.depolarizing(1e-2, 2))
    nzs.add_readout_error(ls.ReadoutError(0.01, 0.03))
    r = ls.run(src, shots=500, seed=11, noise=nzs)
    put("stab_frames64", qasm=src, shots=500, seed=11, counts=r.counts, method=r.method)
    circ = ls.parse(src)
    tab = stab.Tableau(circ.num_qubits)
    for op in circ.operations:
        if op.kind == "gate":
            tab.apply(stab.clifford_map(op.matrix), op.qubits)
    arrays["stab64_x"], arrays["stab64_z"], arrays["stab64_r"] = tab.x, tab.z, tab.r
    x0, basis = tab.copy().support(list(range(64)))
    arrays["stab64_x0"], arrays["stab64_basis"] = x0, basis
    # ideal sampled
    r = ls.run(wl.clifford_layers(30, 5, seed=4), shots=1000, seed=3)
    put("stab_sampled30", qasm=wl.clifford_layers(30, 5, seed=4), shots=1000, seed=3, counts=r.counts,
        method=r.method)
    r = ls.run(PARTIAL_CLIFFORD, shots=800, seed=6, noise=ls.NoiseModel().add_readout_error(0.05))
    put("stab_partial", qasm=PARTIAL_CLIFFORD, shots=800, seed=6, counts=r.counts, method=r.method)
    r = ls.run(DYNAMIC_CLIFFORD, shots=200, seed=2, noise=ls.NoiseModel().add_gate_error(ls.depolarizing(0.05)))
    put("stab_pershot", qasm=DYNAMIC_CLIFFORD, shots=200, seed=2, counts=r.counts, method=r.method)

    # expectations, ideal and noisy
    src = wl.hea(6, 2, seed=5)
    obs = wl.random_pauli_sum(6, 8, seed=1)
    nze = ls.NoiseModel.uniform(single=5e-3, two=2e-2)
    put("expect_hea6", qasm=src, observable=obs, ideal=ls.expectation(src, obs),
        noisy=ls.expectation(src, obs, nze))

    np.savez_compressed(HERE / "golden.npz", **arrays)
    (HERE / "golden.json").write_text(json.dumps(meta, indent=1, sort_keys=True))
    print("wrote", HERE / "golden.npz", HERE / "golden.json")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/lucivant-sim/src")
    main(sys.argv[1])
