"""GPU parity of the statevector and density-matrix engines against the oracle and Orrery's golden
vectors: complex128 to max-abs 1e-12, complex64 to probability TVD 1e-6, counts identical."""

from __future__ import annotations

import numpy as np
import pytest

import lucivant_sim_gb300 as ls
from lucivant_sim_gb300 import _lib, engine, workloads as wl
from lucivant_sim_gb300.noise import NoiseModel, ReadoutError, depolarizing, thermal_relaxation
from lucivant_sim_gb300 import noise as nz
from oracle import dense

pytestmark = pytest.mark.gpu

ATOL_C128 = 1e-12  # max-abs amplitude / probability error of the complex128 path
TVD_C64 = 1e-6  # probability total-variation distance of the complex64 path


def tvd(p: np.ndarray, q: np.ndarray) -> float:
    return 0.5 * float(np.abs(p - q).sum())


@pytest.fixture(params=[None, "7", "8"], ids=["tile-default", "tile7", "tile8"])
def tile_bits(request, monkeypatch):
    if request.param is not None:
        monkeypatch.setenv("LSG_TILE_BITS", request.param)
        monkeypatch.setenv("LSG_LOW_BITS", "3")
    return request.param


@pytest.fixture(params=["ptm", "superop"])
def dm_form(request, monkeypatch):
    """Density matrices in Pauli-transfer form (real, the default) and complex vectorised form."""
    monkeypatch.setenv("LSG_DM_FORM", request.param)
    return request.param


def test_statevector_golden(golden, golden_arrays, tile_bits):
    for case, key in (("sv_bw8", "sv_bw8_state"), ("sv_gates", "sv_gates_state")):
        got = ls.statevector(golden[case]["qasm"])
        assert np.max(np.abs(got - golden_arrays[key])) < ATOL_C128


def test_counts_identical_to_orrery(golden):
    g = golden["sv_bw8"]
    r = ls.run(g["qasm"], shots=g["shots"], seed=g["seed"])
    assert r.method == "statevector" and r.counts == g["counts"]
    assert r.circuit_digest == g["circuit_digest"]
    g = golden["sv_bw8_readout"]
    r = ls.run(g["qasm"], shots=g["shots"], seed=g["seed"], noise=NoiseModel().add_readout_error(ReadoutError(0.05, 0.1)))
    assert r.counts == g["counts"]
    assert ls.verify(r.to_dict(), g["qasm"], NoiseModel().add_readout_error(ReadoutError(0.05, 0.1)))


def _dm_noise():
    return NoiseModel.uniform(single=1e-3, two=1e-2, readout=2e-2).add_gate_error(
        thermal_relaxation(t1=120, t2=90, time=0.05), gates="u3"
    )


def test_density_matrix_golden(golden, golden_arrays, tile_bits, dm_form):
    g = golden["dm_bw4"]
    rho = ls.density_matrix(g["qasm"], _dm_noise())
    assert np.max(np.abs(rho - golden_arrays["dm_bw4_rho"])) < ATOL_C128
    r = ls.run(g["qasm"], shots=g["shots"], seed=g["seed"], noise=_dm_noise())
    assert r.method == "density_matrix" and r.counts == g["counts"]
    for label, want in g["expectations"].items():
        assert abs(ls.expectation(g["qasm"], label, _dm_noise()) - want) < ATOL_C128
    got = ls.outcome_probabilities(g["qasm"], _dm_noise())
    assert got.keys() == g["outcome_probabilities"].keys()
    assert all(abs(got[k] - v) < ATOL_C128 for k, v in g["outcome_probabilities"].items())


def test_every_channel_kind(golden, golden_arrays, dm_form):
    g = golden["dm_channels"]
    noise = (
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
    rho = ls.density_matrix(g["qasm"], noise)
    assert np.max(np.abs(rho - golden_arrays["dm_channels_rho"])) < ATOL_C128
    got = ls.outcome_probabilities(g["qasm"], noise)
    assert got.keys() == g["outcome_probabilities"].keys()
    assert all(abs(got[k] - v) < ATOL_C128 for k, v in g["outcome_probabilities"].items())


OVERLAPPING_PAIRS = """OPENQASM 3.0;
include "stdgates.inc";
qubit[5] q;
bit[6] c;
h q[0]; cx q[0], q[1]; ry(0.9) q[2]; cx q[2], q[3]; rx(0.4) q[4]; cz q[4], q[1];
c[0] = measure q[0];
c[1] = measure q[1];
c[2] = measure q[1];
c[3] = measure q[2];
c[3] = measure q[4];
c[5] = measure q[3];
"""


@pytest.mark.parametrize("noisy", [False, True])
def test_outcome_probabilities_readout_on_device(noisy):
    """Readout branching on the device against the oracle's restatement of Orrery's loop: a qubit
    measured into two classical bits (independent flips), two qubits measured into one classical
    bit (bits combine by OR), a classical bit never written, readout errors on some qubits; on the
    statevector and the density-matrix path."""
    c = ls.parse(OVERLAPPING_PAIRS)
    noise = NoiseModel().add_readout_error(ReadoutError(0.03, 0.07), qubits=[1]).add_readout_error(
        ReadoutError(0.1, 0.02), qubits=[4]).add_readout_error(ReadoutError(0.05, 0.05), qubits=[0])
    if noisy:
        noise.add_gate_error(depolarizing(0.05), gates="h").add_gate_error(depolarizing(0.02, 2), gates="cx")
    want = dense.outcome_probabilities(c, noise)
    got = ls.outcome_probabilities(c, noise)
    assert got.keys() == want.keys()
    assert all(abs(got[k] - v) < ATOL_C128 for k, v in want.items())
    assert abs(sum(got.values()) - 1) < 1e-12


def test_expectation_golden(golden, dm_form):
    g = golden["expect_hea6"]
    assert abs(ls.expectation(g["qasm"], g["observable"]) - g["ideal"]) < ATOL_C128
    assert abs(ls.expectation(g["qasm"], g["observable"], NoiseModel.uniform(single=5e-3, two=2e-2)) - g["noisy"]) < ATOL_C128


@pytest.mark.parametrize("n", [1, 2, 5, 11, 14, 17])
def test_random_brickwork_against_oracle(n, tile_bits):
    src = wl.brickwork(n, 4, seed=100 + n)
    c = ls.parse(src)
    want = dense.evolve_sv(c)
    got = ls.statevector(c)
    assert np.max(np.abs(got - want)) < ATOL_C128
    p = ls.probabilities_array(c)
    assert np.max(np.abs(p - np.abs(want) ** 2)) < ATOL_C128


@pytest.mark.parametrize("n", [3, 7])
def test_noisy_dm_against_oracle(n, tile_bits, dm_form):
    src = wl.brickwork(n, 3, seed=200 + n)
    c = ls.parse(src)
    noise = _dm_noise()
    want = dense.evolve_dm(c, noise).reshape(1 << n, 1 << n)
    got = ls.density_matrix(c, noise)
    assert np.max(np.abs(got - want)) < ATOL_C128


def test_complex64_statevector_tvd():
    c = ls.parse(wl.brickwork(16, 12, seed=5))
    want = np.abs(dense.evolve_sv(c)) ** 2
    got = ls.probabilities_array(c, precision="c64")
    assert tvd(got, want) < TVD_C64


@pytest.mark.parametrize("n", [6, 7])
def test_complex64_density_tvd(dm_form, n):
    """7 qubits: a 14-bit Pauli-transfer register in FP32 takes 2^13-element tiles with two
    register groups per thread."""
    c = ls.parse(wl.brickwork(n, 6, seed=6))
    want = dense.probabilities_array(c, _dm_noise())
    got = ls.probabilities_array(c, _dm_noise(), precision="c64")
    assert tvd(got, want) < TVD_C64


def test_pauli_sums_against_oracle():
    c = ls.parse(wl.hea(9, 3, seed=9))
    obs = wl.random_pauli_sum(9, 20, seed=3)
    assert abs(ls.expectation(c, obs) - dense.expectation(c, obs)) < 1e-11
    noise = NoiseModel.uniform(single=1e-2, two=3e-2)
    c = ls.parse(wl.hea(5, 2, seed=2))
    obs = wl.random_pauli_sum(5, 12, seed=4)
    assert abs(ls.expectation(c, obs, noise) - dense.expectation(c, obs, noise)) < 1e-11


def test_marginal_sampling_matches_oracle():
    src = ls.parse(
        "OPENQASM 3; include \"stdgates.inc\"; qubit[12] q; bit[3] c; bit[2] d;"
        + "".join(f"ry({0.1 + 0.23 * i}) q[{i}];" for i in range(12))
        + "cx q[0], q[5]; cx q[7], q[11]; c[0] = measure q[9]; c[2] = measure q[3]; c[1] = measure q[0];"
        + "d = measure q[10:11]; c[0] = measure q[2];"
    )
    noise = NoiseModel().add_readout_error(ReadoutError(0.1, 0.2), qubits=[3]).add_readout_error(0.05, qubits=[11])
    want, _, _ = dense.run_counts(src, 5000, 17, noise)
    got = ls.run(src, shots=5000, seed=17, noise=noise)
    assert got.counts == want


def test_batched_register_members_are_independent():
    c = ls.parse(wl.brickwork(10, 3, seed=1))
    ops = engine.sv_oplist(c)
    with _lib.Register(10, _lib.C128, batch=3) as reg:
        reg.apply(ops)
        out = reg.download()
    want = dense.evolve_sv(c)
    for b in range(3):
        assert np.max(np.abs(out[b] - want)) < ATOL_C128


def test_batched_noise_instances():
    c = ls.parse(wl.brickwork(4, 2, seed=8, measure=False))
    rng = np.random.default_rng(0)
    noises = [wl.dm_noise(single=float(rng.uniform(1e-4, 5e-3)), two=float(rng.uniform(1e-3, 3e-2))) for _ in range(5)]
    ops = engine.dm_oplist(c, noises)
    with _lib.Register(8, _lib.C128, batch=5) as reg:
        reg.apply(ops)
        out = reg.download()
    for b, nm in enumerate(noises):
        assert np.max(np.abs(out[b] - dense.evolve_dm(c, nm))) < ATOL_C128


def test_density_batch_in_halves_matches_one_batch():
    """run_density_batch evolves an even batch as two halves (the second built while the first
    runs): every member's probabilities and expectations equal the whole batch's bit for bit."""
    from lucivant_sim_gb300.batch import run_density_batch

    c = ls.parse(wl.brickwork(6, 3, seed=12, measure=False))
    noises = wl.dm_noise_instances(8, seed=4)
    labels = wl.z_observables(6)
    p2, e2 = run_density_batch(c, noises, labels, precision="c64", split=True)
    p1, e1 = run_density_batch(c, noises, labels, precision="c64", split=False)
    assert p2.shape == p1.shape == (8, 64) and e2.shape == e1.shape == (len(labels), 8)
    assert np.array_equal(p1, p2) and np.array_equal(e1, e2)
    p3, e3 = run_density_batch(c, noises[:7], labels, precision="c64")  # odd: one batch
    assert np.array_equal(p3, p1[:7]) and np.array_equal(e3, e1[:, :7])


@pytest.mark.parametrize("precision", ["c128", "c64"])
def test_batched_pauli_transfer_instances(precision):
    """Noise instances of one circuit in one Pauli-transfer register: probabilities and Z
    observables of every member against the oracle's density matrix."""
    from lucivant_sim_gb300.batch import DensityBatch

    c = ls.parse(wl.brickwork(5, 4, seed=31, measure=False))
    noises = wl.dm_noise_instances(6, seed=3)
    labels = wl.z_observables(5)
    b = DensityBatch(c, noises, precision=precision)
    try:
        assert b.form == "ptm" and b.reg.real
        b.evolve()
        probs, exps = b.probabilities(), b.expectations(labels)
    finally:
        b.free()
    tol = ATOL_C128 if precision == "c128" else 2e-6
    for i, nm in enumerate(noises):
        want = dense.probabilities_array(c, nm)
        assert (np.max(np.abs(probs[i] - want)) < tol) if precision == "c128" else (tvd(probs[i], want) < TVD_C64)
        for t, lab in enumerate(labels):
            assert abs(exps[t, i] - dense.expectation(c, lab, nm)) < tol


def test_pauli_transfer_register_basics():
    """Basis states, downloads and conversion of a real register; statevector-only calls refuse it."""
    with _lib.Register(6, _lib.R64) as reg:
        reg.set_basis(5)  # |101><101| on 3 qubits
        r = reg.download()[0]
        z = np.arange(8)
        want = np.zeros(64)
        want[:8] = [(-1) ** bin(int(v) & 5).count("1") for v in z]
        assert np.array_equal(r, want)
        rho = engine.density_download(reg)
        expect = np.zeros((8, 8), dtype=np.complex128)
        expect[5, 5] = 1
        assert np.max(np.abs(rho - expect)) < 1e-15
        assert np.allclose(reg.probabilities(3), np.eye(8)[5])
        with pytest.raises(_lib.EngineError, match="statevector register"):
            reg.prob_one(0)
    with pytest.raises(ValueError, match="even number"):
        _lib.Register(5, _lib.R32)


def test_full_size_config1_parity():
    """20 qubits x 20 brickwork layers, 10,000 shots, seed 7: statevector to 1e-12, counts identical."""
    src = wl.brickwork(20, 20, seed=7)
    c = ls.parse(src)
    want_sv = dense.evolve_sv(c)
    r = ls.run(c, shots=10_000, seed=7)
    assert np.max(np.abs(r.statevector - want_sv)) < ATOL_C128
    want_counts = dense.sample(c, np.abs(want_sv) ** 2, 10_000, None, np.random.default_rng(7))
    diff = {k for k in set(want_counts) | set(r.counts) if want_counts.get(k) != r.counts.get(k)}
    # every difference must come from a shot listed as lying on a CDF boundary: such a shot moves
    # from the oracle's outcome to a neighbouring one in CDF order (all 20 qubits are measured in
    # order, so the outcome string read as binary is the CDF index)
    near = r.report.get("near_boundary_shots", [])
    cum = np.cumsum(np.abs(want_sv) ** 2)
    cum /= cum[-1]
    idx = np.searchsorted(cum, np.random.default_rng(7).random(10_000), side="right")
    allowed = {int(idx[s]) + d for s in near for d in (-1, 0, 1)}
    assert {int(k, 2) for k in diff} <= allowed, f"count differences not explained by boundary shots: {sorted(diff)[:8]}"
    moved = sum(abs(want_counts.get(k, 0) - r.counts.get(k, 0)) for k in diff)
    assert moved <= 2 * len(near)
    assert abs(np.vdot(r.statevector, r.statevector).real - 1) < 1e-12


@pytest.mark.parametrize("precision", ["c128", "c64"])
def test_deep_circuit_on_few_qubits(precision):
    """More operators than one pass holds: the plan splits them and the state is unchanged."""
    c = ls.parse(wl.brickwork(10, 150, seed=12))
    want = dense.evolve_sv(c)
    got = ls.statevector(c, precision=precision)
    assert np.max(np.abs(got - want)) < (ATOL_C128 if precision == "c128" else 2e-5)


def test_capacity_errors():
    with pytest.raises(ls.SimulationError, match="up to 26"):
        ls.statevector("OPENQASM 3; qubit[27] q; h q[0];")
    with pytest.raises(ls.SimulationError, match="up to 13"):
        ls.density_matrix("OPENQASM 3; qubit[14] q; h q[0];", NoiseModel.uniform(single=0.01))


@pytest.mark.parametrize("precision", ["c128", "c64"])
@pytest.mark.parametrize("tile", [None, "13"])
def test_wide_operators_on_large_tiles(precision, tile, monkeypatch):
    """Operators wider than a register block (c3x, c4x, ccz, rccx, two-qubit Kraus channels) run
    through the shared-memory path on tiles with more groups than compute threads."""
    if tile:
        monkeypatch.setenv("LSG_TILE_BITS", tile)
    src = ("OPENQASM 3; include \"stdgates.inc\"; qubit[14] q;"
           + "".join(f"u3({0.3 + 0.1 * i}, {0.2 * i}, {0.7 - 0.05 * i}) q[{i}];" for i in range(14))
           + "ccx q[0], q[7], q[13]; c3x q[1], q[5], q[9], q[12]; c4x q[13], q[2], q[4], q[6], q[8];"
           + "ccz q[3], q[10], q[11]; rccx q[12], q[0], q[6]; cswap q[2], q[9], q[1]; cx q[13], q[0];")
    c = ls.parse(src)
    want = dense.evolve_sv(c)
    got = ls.statevector(c, precision=precision)
    tol = ATOL_C128 if precision == "c128" else 1e-5
    assert np.max(np.abs(got - want)) < tol
    dm_src = ("OPENQASM 3; include \"stdgates.inc\"; qubit[6] q;"
              + "".join(f"ry({0.4 + 0.3 * i}) q[{i}]; cx q[{i}], q[{(i + 1) % 6}];" for i in range(6)))
    noise = NoiseModel().add_gate_error(nz.pauli_channel({"XY": 0.05, "ZX": 0.03, "YY": 0.02}), gates="cx")
    cd = ls.parse(dm_src)
    want = dense.evolve_dm(cd, noise).reshape(64, 64)
    got = ls.density_matrix(cd, noise, precision=precision)
    assert np.max(np.abs(got - want)) < tol


@pytest.mark.parametrize("noisy", [False, True])
def test_precision_report_matches_the_oracle(noisy):
    """The complex64 path's reported errors (against a complex128 re-run on the device) are the
    errors against the FP64 oracle: the complex128 path equals the oracle to 1e-12."""
    n = 5 if noisy else 10
    c = ls.parse(wl.brickwork(n, 4, seed=21, measure=False))
    noise = _dm_noise() if noisy else None
    rep = ls.precision_report(c, noise)
    zs = wl.z_observables(n)[:n]
    if noisy:
        got_state = ls.density_matrix(c, noise, precision="c64")
        want_state = dense.evolve_dm(c, noise).reshape(1 << n, 1 << n)
        want_p = dense.probabilities_array(c, noise)
    else:
        got_state = ls.statevector(c, precision="c64")
        want_state = dense.evolve_sv(c)
        want_p = np.abs(want_state) ** 2
    got_p = ls.probabilities_array(c, noise, precision="c64")
    want_amp = float(np.max(np.abs(got_state - want_state)))
    want_tvd = 0.5 * float(np.abs(got_p - want_p).sum())
    want_exp = max(abs(ls.expectation(c, z, noise, precision="c64") - dense.expectation(c, z, noise)) for z in zs)
    assert abs(rep["max_amplitude_error"] - want_amp) < 1e-12
    assert abs(rep["probability_tvd"] - want_tvd) < 1e-12
    assert abs(rep["expectation_error"] - want_exp) < 1e-12
    assert 0 < rep["probability_tvd"] < 1e-6
    r = ls.run(wl.brickwork(n, 4, seed=21), shots=100, seed=3, noise=noise, precision="c64", report_precision=True)
    assert abs(r.report["precision"]["probability_tvd"] - rep["probability_tvd"]) < 1e-15
    assert "precision" not in ls.run(wl.brickwork(n, 4, seed=21), shots=100, seed=3, noise=noise).report
