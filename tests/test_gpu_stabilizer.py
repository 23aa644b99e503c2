"""The stabilizer engine on the GPU: tableaux, support and counts bit-exact against Orrery's
golden vectors and the oracle."""

from __future__ import annotations

import numpy as np
import pytest

import lucivant_sim_gb300 as ls
from lucivant_sim_gb300 import stabilizer as st, workloads as wl
from lucivant_sim_gb300.clifford import all_gates
from lucivant_sim_gb300.noise import NoiseModel, ReadoutError, depolarizing
from oracle import tableau

pytestmark = pytest.mark.gpu


def _tab(circuit):
    enc = st.Encoder(None)
    t = st.Tableau(circuit.num_qubits)
    t.apply(enc.encode(all_gates(circuit.operations), False), enc)
    return t


def test_tableau_and_support_golden(golden, golden_arrays):
    c = ls.parse(golden["stab_frames64"]["qasm"])
    t = _tab(c)
    x, z, r = t.arrays()
    assert np.array_equal(x, golden_arrays["stab64_x"])
    assert np.array_equal(z, golden_arrays["stab64_z"])
    assert np.array_equal(r, golden_arrays["stab64_r"])
    x0, basis = t.support(list(range(64)))
    assert np.array_equal(x0, golden_arrays["stab64_x0"])
    assert np.array_equal(basis, golden_arrays["stab64_basis"])
    t.free()


@pytest.mark.parametrize("n,layers,seed", [(5, 6, 1), (37, 5, 2), (130, 3, 3)])
def test_tableau_generic_gates_against_oracle(n, layers, seed):
    rng = np.random.default_rng(seed)
    lines = ["OPENQASM 3.0;", 'include "stdgates.inc";', f"qubit[{n}] q;"]
    names1 = ["h", "s", "sdg", "x", "y", "z", "sx", "sxdg", "id"]
    names2 = ["cx", "cz", "cy", "swap", "iswap", "ecr", "dcx"]
    for _ in range(layers):
        for q in range(n):
            lines.append(f"{names1[rng.integers(len(names1))]} q[{q}];")
        perm = rng.permutation(n)
        for i in range(0, n - 1, 2):
            lines.append(f"{names2[rng.integers(len(names2))]} q[{perm[i]}], q[{perm[i + 1]}];")
    c = ls.parse("\n".join(lines))
    ref = tableau.reference_tableau(c)
    t = _tab(c)
    x, z, r = t.arrays()
    assert np.array_equal(x, ref.x) and np.array_equal(z, ref.z) and np.array_equal(r, ref.r)
    qs = sorted(rng.choice(n, size=max(1, n // 3), replace=False).tolist())
    want_x0, want_basis = ref.copy().support(qs)
    x0, basis = t.support(qs)
    assert np.array_equal(x0, want_x0) and np.array_equal(basis, want_basis)
    t.free()


def _partial_clifford(n: int, layers: int, seed: int, frac: float):
    """Random h/s/cx/cz layers on a random fraction of the qubits: the rest stay |0>, so both
    the X pivots and the Z constraints of support() have work."""
    rng = np.random.default_rng(seed)
    active = rng.permutation(n)[: max(1, int(frac * n))]
    lines = ["OPENQASM 3.0;", 'include "stdgates.inc";', f"qubit[{n}] q;"]
    for _ in range(layers):
        for q in active:
            lines.append(f"{['h', 's', 'x', 'sdg'][rng.integers(4)]} q[{q}];")
        perm = rng.permutation(active)
        for i in range(0, len(perm) - 1, 2):
            lines.append(f"{['cx', 'cz'][rng.integers(2)]} q[{perm[i]}], q[{perm[i + 1]}];")
    return ls.parse("\n".join(lines))


@pytest.mark.parametrize("n,frac", [(1, 1.0), (2, 0.5), (63, 0.7), (64, 1.0), (65, 0.3), (257, 0.6), (1000, 0.5), (2048, 0.8)])
def test_support_one_launch_equals_launch_per_column(n, frac, monkeypatch):
    """support() in one cluster launch (rows in distributed shared memory) against the path with a
    launch per column, on full and partial qubit subsets; against the oracle up to 130 qubits."""
    c = _partial_clifford(n, 4, seed=n, frac=frac)
    rng = np.random.default_rng(n + 1)
    subsets = [list(range(n)), sorted(rng.choice(n, size=max(1, n // 3), replace=False).tolist())]
    t = _tab(c)
    try:
        got = [t.support(qs) for qs in subsets]
        monkeypatch.setenv("LSG_SUPPORT_STEPS", "1")
        want = [t.support(qs) for qs in subsets]
    finally:
        t.free()
    for (x0, basis), (wx0, wbasis) in zip(got, want):
        assert np.array_equal(x0, wx0) and np.array_equal(basis, wbasis)
    if n <= 130:
        ref = tableau.reference_tableau(c)
        for qs, (x0, basis) in zip(subsets, got):
            rx0, rbasis = ref.copy().support(qs)
            assert np.array_equal(x0, rx0) and np.array_equal(basis, rbasis)


def test_counts_golden(golden):
    g = golden["stab_frames64"]
    noise = NoiseModel()
    noise.add_gate_error(depolarizing(1e-2, 1)).add_gate_error(depolarizing(1e-2, 2))
    noise.add_readout_error(ReadoutError(0.01, 0.03))
    r = ls.run(g["qasm"], shots=g["shots"], seed=g["seed"], noise=noise)
    assert r.method == "stabilizer" and r.counts == g["counts"]
    g = golden["stab_sampled30"]
    assert ls.run(g["qasm"], shots=g["shots"], seed=g["seed"]).counts == g["counts"]
    g = golden["stab_partial"]
    assert ls.run(g["qasm"], shots=g["shots"], seed=g["seed"], noise=NoiseModel().add_readout_error(0.05)).counts == g["counts"]


def test_frames_against_oracle_and_rng_position():
    c = wl.clifford_layers_circuit(100, 6, seed=9)
    noise = wl.stabilizer_noise(2e-2)
    rng_a = np.random.default_rng(21)
    want = tableau.frames(c, 333, noise, rng_a)
    rng_b = np.random.default_rng(21)
    got = st.frames(c, 333, noise, rng_b)
    assert got == want
    assert rng_b.bit_generator.state == rng_a.bit_generator.state


def test_sampled_against_oracle_and_rng_position():
    c = ls.parse(wl.clifford_layers(45, 4, seed=8))
    rng_a = np.random.default_rng(5)
    want = tableau.sampled(c, 701, NoiseModel().add_readout_error(0.1), rng_a)
    rng_b = np.random.default_rng(5)
    got = st.sampled(c, 701, NoiseModel().add_readout_error(0.1), rng_b)
    assert got == want
    assert rng_b.bit_generator.state == rng_a.bit_generator.state


def test_per_shot_golden_and_oracle(golden):
    g = golden["stab_pershot"]
    noise = NoiseModel().add_gate_error(depolarizing(0.05))
    assert ls.run(g["qasm"], shots=g["shots"], seed=g["seed"], noise=noise).counts == g["counts"]
    # more shapes against the oracle, with readout and the generator's final state
    src = g["qasm"].replace("c = measure q;", "c[3] = measure q[3]; if (c[3] == 1) { x q[5]; } else { h q[5]; }\nc = measure q;")
    c = ls.parse(src)
    noise = NoiseModel().add_gate_error(depolarizing(0.1)).add_gate_error(depolarizing(0.05, 2))
    noise.add_readout_error(ReadoutError(0.02, 0.05))
    from lucivant_sim_gb300 import stabilizer_shots

    rng_a = np.random.default_rng(77)
    want = tableau.per_shot(c, 150, noise, rng_a)
    rng_b = np.random.default_rng(77)
    got = stabilizer_shots.per_shot(c, 150, noise, rng_b)
    assert got == want
    assert rng_b.bit_generator.state == rng_a.bit_generator.state
