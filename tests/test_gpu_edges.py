"""Edge cases of the device engines: empty circuits, zero shots, one qubit, the largest registers
(26-qubit statevector, 13-qubit density matrix), parameter binding, and the probability API's
threshold."""

from __future__ import annotations

import numpy as np
import pytest

import lucivant_sim_gb300 as ls
from lucivant_sim_gb300 import workloads as wl
from lucivant_sim_gb300.noise import NoiseModel
from oracle import dense

pytestmark = pytest.mark.gpu


def test_empty_circuit_and_zero_shots():
    sv = ls.statevector("OPENQASM 3; qubit[3] q;")
    assert sv[0] == 1 and np.count_nonzero(sv) == 1
    r = ls.run("OPENQASM 3; qubit[2] q; bit[2] c; c = measure q;", shots=0, seed=1)
    assert r.counts == {} and r.shots == 0
    r = ls.run("OPENQASM 3; qubit[2] q; bit[2] c; c = measure q;", shots=50, seed=1)
    assert r.counts == {"00": 50}
    rho = ls.density_matrix("OPENQASM 3; qubit[2] q;", NoiseModel.uniform(single=0.1))
    assert rho[0, 0] == pytest.approx(1.0, abs=1e-15) and np.count_nonzero(np.abs(rho) > 1e-15) == 1


def test_one_qubit():
    src = 'OPENQASM 3; include "stdgates.inc"; qubit[1] q; bit[1] c; h q[0]; c[0] = measure q[0];'
    want, _, _ = dense.run_counts(ls.parse(src), 1000, 3)
    assert ls.run(src, shots=1000, seed=3).counts == want
    noise = NoiseModel.uniform(single=0.2, readout=0.1)
    want, _, _ = dense.run_counts(ls.parse(src), 1000, 3, noise)
    assert ls.run(src, shots=1000, seed=3, noise=noise).counts == want


@pytest.mark.parametrize("precision", ["c64", "c128"])
def test_largest_statevector(precision):
    """26 qubits (Orrery's limit): h on every qubit, then a phase on the last; every amplitude is
    ±2^-13."""
    src = 'OPENQASM 3; include "stdgates.inc"; qubit[26] q; h q; z q[25];'
    sv = ls.statevector(src, precision=precision)
    tol = 1e-12 if precision == "c128" else 1e-7
    assert sv.shape == (1 << 26,)
    assert np.max(np.abs(np.abs(sv) - 2.0**-13)) < tol
    assert np.all(sv[: 1 << 25].real > 0) and np.all(sv[1 << 25 :].real < 0)


@pytest.mark.parametrize("form", ["ptm", "superop"])
def test_largest_density_matrix(form, monkeypatch):
    """13 qubits (Orrery's density-matrix limit), noiseless: rho's diagonal is the statevector's
    probabilities."""
    monkeypatch.setenv("LSG_DM_FORM", form)
    c = ls.parse(wl.brickwork(13, 2, seed=9, measure=False))
    want = np.abs(dense.evolve_sv(c)) ** 2
    # a noise model with a channel that never fires keeps the density-matrix method
    quiet = NoiseModel().add_gate_error(ls.depolarizing(0.0), gates="id")
    got = ls.probabilities_array(c, quiet)
    assert np.max(np.abs(got - want)) < 1e-12


def test_parameters_and_thresholded_probabilities():
    src = 'OPENQASM 3; include "stdgates.inc"; input float t; qubit[2] q; ry(t) q[0]; cx q[0], q[1];'
    probs = ls.probabilities(src, params={"t": np.pi / 3})
    assert set(probs) == {"00", "11"}
    assert probs["11"] == pytest.approx(np.sin(np.pi / 6) ** 2, abs=1e-12)
    assert ls.probabilities(src, params={"t": 0.0}) == {"00": pytest.approx(1.0, abs=1e-12)}
    with pytest.raises(Exception):
        ls.statevector(src)  # the input is unbound


def test_expectations_of_more_members_than_one_launch_takes():
    """70,000 members (above the 65,535 a launch's grid y holds): lsg_expect_pauli splits them
    into launches and every member's expectations equal a host computation from its amplitudes,
    for a complex128 statevector register and a real Pauli-transfer register."""
    from lucivant_sim_gb300 import _lib

    members, n = 70_000, 3
    rng = np.random.default_rng(11)
    vec = rng.normal(size=(members, 1 << n)) + 1j * rng.normal(size=(members, 1 << n))
    vec /= np.linalg.norm(vec, axis=1, keepdims=True)
    xs, zs = [0, 1, 3, 5, 6], [1, 0, 3, 4, 6]
    idx = np.arange(1 << n)
    want = np.empty((len(xs), members))
    for t, (x, z) in enumerate(zip(xs, zs, strict=True)):
        sign = 1.0 - 2.0 * (np.array([bin(i & z).count("1") for i in idx]) & 1)
        phase = 1j ** (bin(x & z).count("1") & 3)
        want[t] = np.real(phase * np.sum(np.conj(vec[:, idx ^ x]) * vec * sign, axis=1))
    with _lib.Register(n, _lib.C128, batch=members) as reg:
        reg.upload(vec)
        got = reg.expect(0, xs, zs)
    assert got.shape == (len(xs), members)
    assert np.max(np.abs(got - want)) < 1e-12
    # Pauli-transfer members: each expectation is the coefficient at the term's digits
    coef = rng.uniform(-1, 1, size=(members, 1 << (2 * n)))
    digits = [(x << n) | z for x, z in zip(xs, zs, strict=True)]
    with _lib.Register(2 * n, _lib.R64, batch=members) as reg:
        reg.upload(coef)
        got = reg.expect(n, xs, zs)
    assert np.array_equal(got, coef[:, digits].T)
