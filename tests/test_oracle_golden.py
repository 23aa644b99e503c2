"""Pin the CPU oracle and the host-side IR against vectors produced by Orrery 0.3.0 itself
(``tests/golden/make_golden.py``) and against Orrery's own known-answer tests."""

from __future__ import annotations

import math

import numpy as np
import pytest

from lucivant_sim_gb300 import qasm
from lucivant_sim_gb300.noise import NoiseModel, ReadoutError, depolarizing, thermal_relaxation
from lucivant_sim_gb300 import noise as nz
from oracle import dense, tableau

TOL = 1e-12


def _parse(src: str):
    return qasm.parse(src)


def test_statevector_brickwork(golden, golden_arrays):
    c = _parse(golden["sv_bw8"]["qasm"])
    assert c.digest() == golden["sv_bw8"]["circuit_digest"]
    v = dense.evolve_sv(c)
    assert np.max(np.abs(v - golden_arrays["sv_bw8_state"])) < TOL


def test_every_gate(golden, golden_arrays):
    v = dense.evolve_sv(_parse(golden["sv_gates"]["qasm"]))
    assert np.max(np.abs(v - golden_arrays["sv_gates_state"])) < TOL


def test_statevector_counts_are_identical(golden):
    g = golden["sv_bw8"]
    counts, method, _ = dense.run_counts(_parse(g["qasm"]), g["shots"], g["seed"])
    assert method == g["method"] and counts == g["counts"]
    g = golden["sv_bw8_readout"]
    noise = NoiseModel().add_readout_error(ReadoutError(0.05, 0.1))
    counts, _, _ = dense.run_counts(_parse(g["qasm"]), g["shots"], g["seed"], noise)
    assert counts == g["counts"]


def _dm_noise():
    return NoiseModel.uniform(single=1e-3, two=1e-2, readout=2e-2).add_gate_error(
        thermal_relaxation(t1=120, t2=90, time=0.05), gates="u3"
    )


def test_density_matrix_and_counts(golden, golden_arrays):
    g = golden["dm_bw4"]
    c = _parse(g["qasm"])
    noise = _dm_noise()
    assert noise.digest() == g["noise_digest"]
    rho = dense.evolve_dm(c, noise).reshape(16, 16)
    assert np.max(np.abs(rho - golden_arrays["dm_bw4_rho"])) < TOL
    counts, method, _ = dense.run_counts(c, g["shots"], g["seed"], noise)
    assert method == "density_matrix" and counts == g["counts"]
    for label, want in g["expectations"].items():
        assert abs(dense.expectation(c, label, noise) - want) < TOL
    got = dense.outcome_probabilities(c, noise)
    assert got.keys() == g["outcome_probabilities"].keys()
    assert all(abs(got[k] - v) < TOL for k, v in g["outcome_probabilities"].items())


def _channel_noise():
    return (
        NoiseModel()
        .add_gate_error(nz.amplitude_damping(0.1), gates="h")
        .add_gate_error(nz.phase_damping(0.2), gates="ry")
        .add_gate_error(nz.bit_flip(0.05), gates="t")
        .add_gate_error(nz.phase_flip(0.07), gates="sx")
        .add_gate_error(nz.pauli_channel({"XY": 0.03, "ZZ": 0.02, "IX": 0.01}), gates="cx")
        .add_gate_error(depolarizing(0.2, 2), gates="cz")
        .add_gate_error(thermal_relaxation(50, 40, 3.0), qubits=[2])
        .add_readout_error(ReadoutError(0.02, 0.04), qubits=[0])
    )


def test_every_channel_kind(golden, golden_arrays):
    g = golden["dm_channels"]
    c = _parse(g["qasm"])
    rho = dense.evolve_dm(c, _channel_noise()).reshape(16, 16)
    assert np.max(np.abs(rho - golden_arrays["dm_channels_rho"])) < TOL
    got = dense.outcome_probabilities(c, _channel_noise())
    assert all(abs(got[k] - v) < TOL for k, v in g["outcome_probabilities"].items())


def test_trajectory_counts_are_identical(golden):
    g = golden["traj_mid8"]
    counts, method, _ = dense.run_counts(_parse(g["qasm"]), g["shots"], g["seed"],
                                         NoiseModel.uniform(single=2e-2, two=5e-2, readout=3e-2))
    assert method == "trajectories" and counts == g["counts"]
    g = golden["traj_mid8_ideal"]
    counts, _, _ = dense.run_counts(_parse(g["qasm"]), g["shots"], g["seed"])
    assert counts == g["counts"]
    g = golden["traj_kraus"]
    counts, _, _ = dense.run_counts(_parse(g["qasm"]), g["shots"], g["seed"],
                                    NoiseModel().add_gate_error(thermal_relaxation(20, 15, 4.0), gates="u3"),
                                    method="trajectories")
    assert counts == g["counts"]


def test_tableau_and_support_bit_exact(golden, golden_arrays):
    c = _parse(golden["stab_frames64"]["qasm"])
    t = tableau.reference_tableau(c)
    assert np.array_equal(t.x, golden_arrays["stab64_x"])
    assert np.array_equal(t.z, golden_arrays["stab64_z"])
    assert np.array_equal(t.r, golden_arrays["stab64_r"])
    x0, basis = t.copy().support(list(range(64)))
    assert np.array_equal(x0, golden_arrays["stab64_x0"])
    assert np.array_equal(basis, golden_arrays["stab64_basis"])


def test_stabilizer_counts_are_identical(golden):
    g = golden["stab_frames64"]
    noise = NoiseModel()
    noise.add_gate_error(depolarizing(1e-2, 1)).add_gate_error(depolarizing(1e-2, 2))
    noise.add_readout_error(ReadoutError(0.01, 0.03))
    counts, method, _ = dense.run_counts(_parse(g["qasm"]), g["shots"], g["seed"], noise)
    assert method == "stabilizer" and counts == g["counts"]
    g = golden["stab_sampled30"]
    counts, method, _ = dense.run_counts(_parse(g["qasm"]), g["shots"], g["seed"])
    assert method == "stabilizer" and counts == g["counts"]
    g = golden["stab_partial"]
    counts, _, _ = dense.run_counts(_parse(g["qasm"]), g["shots"], g["seed"], NoiseModel().add_readout_error(0.05))
    assert counts == g["counts"]
    g = golden["stab_pershot"]
    counts, _, _ = dense.run_counts(_parse(g["qasm"]), g["shots"], g["seed"],
                                    NoiseModel().add_gate_error(depolarizing(0.05)))
    assert counts == g["counts"]


def test_expectation(golden):
    g = golden["expect_hea6"]
    c = _parse(g["qasm"])
    assert abs(dense.expectation(c, g["observable"]) - g["ideal"]) < TOL
    assert abs(dense.expectation(c, g["observable"], NoiseModel.uniform(single=5e-3, two=2e-2)) - g["noisy"]) < TOL


# Orrery's own known answers (tests/test_sim.py:191-218, tests/test_stabilizer.py:97-103)

BELL = 'OPENQASM 3;\ninclude "stdgates.inc";\nqubit[2] q;\nbit[2] c;\nh q[0];\ncx q[0], q[1];\nc = measure q;\n'


def test_known_expectation_xx_under_depolarizing():
    noise = NoiseModel().add_gate_error(depolarizing(0.2, 2), gates="cx")
    assert dense.expectation(_parse(BELL), "XX", noise) == pytest.approx(0.8, abs=1e-12)


def test_known_thermal_decay():
    src = "OPENQASM 3; qubit q; x q;"
    noise = NoiseModel().add_gate_error(nz.amplitude_damping(1 - math.exp(-0.3)), gates="x")
    p = dense.probabilities_array(_parse(src), noise)
    assert p[1] == pytest.approx(math.exp(-0.3), abs=1e-12)


def test_known_reset_and_if():
    c = _parse("OPENQASM 3; qubit q; bit c; x q; reset q; c = measure q;")
    assert dense.run_counts(c, 100, 1)[0] == {"0": 100}
    c = _parse("OPENQASM 3; qubit[2] q; bit[2] c; x q[0]; c[0] = measure q[0]; if (c[0] == 1) x q[1]; "
               "c[1] = measure q[1];")
    assert dense.run_counts(c, 50, 1)[0] == {"11": 50}


def test_known_endianness_of_registers():
    c = _parse("OPENQASM 3; qubit[3] q; bit[1] a; bit[2] b; x q[1]; a[0] = measure q[0]; b = measure q[1:2];")
    counts, method, _ = dense.run_counts(c, 50, 3)
    assert counts == {"01 0": 50}


def test_exact_trajectory_outcomes_explain_orreys_counts(golden):
    """The oracle's exact outcome distribution of a noisy mid-circuit program against Orrery's
    300 recorded shots (chi-square over outcomes expected 5 times or more, pooled tail), and
    against 2,000 shots of the oracle's own trajectories."""
    from scipy.stats import chi2

    g = golden["traj_mid8"]
    c = qasm.parse(g["qasm"])
    noise = NoiseModel.uniform(single=2e-2, two=5e-2, readout=3e-2)
    exact = dense.exact_outcomes(c, noise)
    assert abs(sum(exact.values()) - 1) < 1e-12

    def pvalue(counts: dict[int, int]) -> float:
        shots = sum(counts.values())
        stat, bins, po, pe = 0.0, 0, 0, 0.0
        for k in set(exact) | set(counts):
            e, o = shots * exact.get(k, 0.0), counts.get(k, 0)
            if e >= 5:
                stat, bins = stat + (o - e) ** 2 / e, bins + 1
            else:
                po, pe = po + o, pe + e
        if pe > 0:
            stat, bins = stat + (po - pe) ** 2 / pe, bins + 1
        return float(chi2.sf(stat, max(bins - 1, 1)))

    orrery = {int(k.replace(" ", ""), 2): v for k, v in g["counts"].items()}
    assert pvalue(orrery) > 1e-4
    rng = np.random.default_rng(5)
    own: dict[int, int] = {}
    for _ in range(2000):
        b = dense.trajectory(c, noise, rng)
        own[b] = own.get(b, 0) + 1
    assert pvalue(own) > 1e-4
