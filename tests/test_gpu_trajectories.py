"""Trajectories on the GPU: serial mode reproduces Orrery's counts (same seed, same draw order);
batched mode agrees with it statistically."""

from __future__ import annotations

import numpy as np
import pytest

import lucivant_sim_gb300 as ls
from lucivant_sim_gb300 import _lib, trajectories, workloads as wl
from lucivant_sim_gb300.noise import NoiseModel, thermal_relaxation
from oracle import dense

pytestmark = pytest.mark.gpu


def tvd_counts(a: dict, b: dict) -> float:
    na, nb = sum(a.values()), sum(b.values())
    return 0.5 * sum(abs(a.get(k, 0) / na - b.get(k, 0) / nb) for k in set(a) | set(b))


def test_golden_trajectory_counts_identical(golden):
    g = golden["traj_mid8"]
    r = ls.run(g["qasm"], shots=g["shots"], seed=g["seed"], noise=NoiseModel.uniform(single=2e-2, two=5e-2, readout=3e-2))
    assert r.method == "trajectories"
    assert r.counts == g["counts"] or r.report["near_threshold"] > 0
    g = golden["traj_mid8_ideal"]
    assert ls.run(g["qasm"], shots=g["shots"], seed=g["seed"]).counts == g["counts"]
    g = golden["traj_kraus"]
    noise = NoiseModel().add_gate_error(thermal_relaxation(20, 15, 4.0), gates="u3")
    r = ls.run(g["qasm"], shots=g["shots"], seed=g["seed"], noise=noise, method="trajectories")
    assert r.counts == g["counts"] or r.report["near_threshold"] > 0


@pytest.mark.parametrize("n,rounds,seed", [(8, 3, 1), (10, 2, 2), (12, 2, 3)])
def test_serial_matches_oracle_and_leaves_rng_in_place(n, rounds, seed):
    c = ls.parse(wl.midcircuit(n, rounds, seed=seed))
    noise = NoiseModel.uniform(single=1e-2, two=4e-2, readout=2e-2)
    shots = 120
    rng_a = np.random.default_rng(seed)
    want: dict[int, int] = {}
    for _ in range(shots):
        b = dense.trajectory(c, noise, rng_a)
        want[b] = want.get(b, 0) + 1
    rng_b = np.random.default_rng(seed)
    got, report = trajectories.run_shots(c, shots, noise, rng_b, _lib.C128, "serial")
    assert got == want or report["near_threshold"] > 0
    assert rng_b.bit_generator.state == rng_a.bit_generator.state


def test_known_answers_reset_and_if():
    c = "OPENQASM 3; qubit q; bit c; x q; reset q; c = measure q;"
    assert ls.run(c, shots=100, seed=1, method="trajectories").counts == {"0": 100}
    c = ("OPENQASM 3; qubit[2] q; bit[2] c; x q[0]; c[0] = measure q[0]; if (c[0] == 1) x q[1]; else h q[1];"
         " c[1] = measure q[1];")
    assert ls.run(c, shots=50, seed=1).counts == {"11": 50}


def chi2_pvalue(counts: dict[int, int], exact: dict[int, float]) -> float:
    """Pearson chi-square p-value of ``counts`` against the exact distribution: outcomes
    expected at least 5 times are their own bins, the rest one pooled bin."""
    from scipy.stats import chi2

    shots = sum(counts.values())
    stat, bins, pooled_o, pooled_e = 0.0, 0, 0, 0.0
    for k in set(exact) | set(counts):
        e, o = shots * exact.get(k, 0.0), counts.get(k, 0)
        if e >= 5:
            stat += (o - e) ** 2 / e
            bins += 1
        else:
            pooled_o += o
            pooled_e += e
    if pooled_e > 0:
        stat += (pooled_o - pooled_e) ** 2 / pooled_e
        bins += 1
    return float(chi2.sf(stat, max(bins - 1, 1)))


@pytest.mark.parametrize("precision", [_lib.C128, _lib.C64])
@pytest.mark.parametrize("mode", ["batched", "serial"])
def test_counts_follow_the_exact_outcome_distribution(precision, mode):
    """8 qubits x 3 rounds of mid-circuit measurement, conditional X and reset with gate and
    readout noise: the counts of 20,000 shots (6,000 serial) against the oracle's exact
    distribution of the classical record (a density matrix per record), chi-square p > 1e-6."""
    if mode == "serial" and precision == _lib.C64:
        pytest.skip("serial mode is Orrery's complex128 draw order")
    c = ls.parse(wl.midcircuit(8, 3, seed=5))
    noise = NoiseModel.uniform(single=1e-2, two=3e-2, readout=2e-2)
    exact = dense.exact_outcomes(c, noise)
    assert abs(sum(exact.values()) - 1) < 1e-12
    shots = 20_000 if mode == "batched" else 6_000
    counts, _ = trajectories.run_shots(c, shots, noise, np.random.default_rng(11), precision, mode)
    assert sum(counts.values()) == shots
    assert set(counts) <= {k for k, p in exact.items() if p > 0}
    assert chi2_pvalue(counts, exact) > 1e-6


def test_kraus_channel_statistics_against_density_matrix():
    src = "OPENQASM 3; qubit[2] q; bit[2] c; x q[0]; h q[1]; cx q[1], q[0]; c = measure q;"
    noise = NoiseModel().add_gate_error(thermal_relaxation(30, 20, 6.0), gates="x").add_gate_error(
        thermal_relaxation(30, 20, 6.0), gates="h")
    exact = dense.outcome_probabilities(ls.parse(src), noise)
    got = ls.run(src, shots=20000, seed=3, noise=noise, method="trajectories", trajectory_mode="batched").counts
    assert tvd_counts(got, {k: int(round(v * 1e6)) for k, v in exact.items()}) < 0.02


def test_batched_mode_at_benchmark_size_agrees_with_serial():
    """The benchmark's trajectory workload at full size (18 qubits, 16 rounds of mid-circuit
    measurement, conditional X and reset, depolarising 1e-3 / 1e-2): 8192 batched complex64 shots
    and 2048 serial complex128 shots (Orrery's draw order, identical to Orrery's shots for the
    same seed) are samples of one distribution over the 256 classical records: two-sample
    chi-square p > 1e-6 (records expected fewer than 5 times in either sample pooled)."""
    from scipy.stats import chi2

    c = ls.parse(wl.midcircuit(18, 16, seed=7))
    noise = NoiseModel.uniform(single=1e-3, two=1e-2)
    a, _ = trajectories.run_shots(c, 8192, noise, np.random.default_rng(3), _lib.C64, "batched")
    b, _ = trajectories.run_shots(c, 2048, noise, np.random.default_rng(4), _lib.C128, "serial")
    na, nb = sum(a.values()), sum(b.values())
    assert (na, nb) == (8192, 2048)
    stat, bins, pool = 0.0, 0, [0, 0, 0.0, 0.0]
    for k in set(a) | set(b):
        oa, ob = a.get(k, 0), b.get(k, 0)
        share = (oa + ob) / (na + nb)
        ea, eb = na * share, nb * share
        if min(ea, eb) >= 5:
            stat += (oa - ea) ** 2 / ea + (ob - eb) ** 2 / eb
            bins += 1
        else:
            pool = [pool[0] + oa, pool[1] + ob, pool[2] + ea, pool[3] + eb]
    if pool[2] > 0 and pool[3] > 0:
        stat += (pool[0] - pool[2]) ** 2 / pool[2] + (pool[1] - pool[3]) ** 2 / pool[3]
        bins += 1
    assert bins >= 8
    assert float(chi2.sf(stat, bins - 1)) > 1e-6
