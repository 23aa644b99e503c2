"""The CUDA path against Orrery at the benchmarked sizes (``tests/golden/configs.*``, made by
running Orrery 0.3.0 itself on the same seeded workloads).

* 12-qubit, 12-layer noisy density matrices: the benchmark's 256-instance batch in the real64
  Pauli-transfer register and in double-float pairs (instances 0, 1, 128, 255 to a max-abs error of
  1e-12 on the 4096 probabilities and the 23 <Z> observables), the same batch in real32
  (probability TVD <= 1e-6),
  and Orrery's own noise reading through the public API in both register forms (1e-12).
* 18 qubits x 16 rounds of mid-circuit measurement: 64 shots in Orrery's draw order give
  Orrery's counts and leave the generator where Orrery leaves it.
* 2048 qubits x 1000 Clifford layers with Pauli noise: the tableau, x0, the row basis and the
  counts of 1000 shots are bit-exact.
* Every Clifford gate name on a 6-qubit tableau: bit-exact.
"""

from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import lucivant_sim_gb300 as ls
from lucivant_sim_gb300 import _lib, stabilizer as st, trajectories, workloads as wl
from lucivant_sim_gb300.batch import DensityBatch
from lucivant_sim_gb300.clifford import all_gates
from lucivant_sim_gb300.noise import NoiseModel

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
ATOL_F64 = 1e-12  # the complex128 path's tolerance: max-abs on probabilities and expectations
TVD_F32 = 1e-6  # the complex64 request's tolerance: probability total-variation distance
ZTOL_F32 = 1e-5  # and its expectations, max-abs


@pytest.fixture(scope="module")
def cfg() -> dict:
    path = GOLDEN / "configs.json"
    if not path.exists():
        pytest.skip("benchmark-size fixtures not generated")
    return json.loads(path.read_text())["cases"]


@pytest.fixture(scope="module")
def cfg_arrays() -> dict:
    with np.load(GOLDEN / "configs.npz") as data:
        return {k: data[k] for k in data.files}


def _members(cfg) -> list[int]:
    return sorted(int(k[len("cfg2_inst"):]) for k in cfg if k.startswith("cfg2_inst"))


@pytest.mark.parametrize("precision", ["c128", "df64", "c64"])
def test_benchmark_batch_members_match_orrery(cfg, cfg_arrays, precision):
    """The benchmark's step itself: 256 instances in one register, every member evolved by the
    specialized passes, reduced on the device; the fixture members compared with Orrery's."""
    circuit = ls.parse(wl.brickwork(12, 12, seed=7, measure=False))
    noises = wl.dm_noise_instances(256, seed=7)
    labels = wl.z_observables(12)
    b = DensityBatch(circuit, noises, precision=precision)
    try:
        b.evolve()
        probs = b.probabilities()
        exps = b.expectations(labels)
    finally:
        b.free()
    for m in _members(cfg):
        want_p = cfg_arrays[f"cfg2_inst{m}_probs"]
        want_z = np.asarray(cfg[f"cfg2_inst{m}"]["z"])
        if precision in ("c128", "df64"):  # double-float pairs are held to the FP64 tolerance
            assert np.max(np.abs(probs[m] - want_p)) < ATOL_F64, m
            assert np.max(np.abs(exps[:, m] - want_z)) < ATOL_F64, m
        else:
            assert 0.5 * np.abs(probs[m] - want_p).sum() < TVD_F32, m
            assert np.max(np.abs(exps[:, m] - want_z)) < ZTOL_F32, m


@pytest.mark.parametrize("form", ["ptm", "superop"])
def test_orrery_noise_reading_through_the_api(cfg, cfg_arrays, form, monkeypatch):
    """Orrery's own reading of "uniform noise plus thermal relaxation on u3" (the thermal rule
    replaces the depolarising one on u3) through ls.probabilities_array and ls.expectation, in the
    Pauli-transfer and the complex vectorised register."""
    monkeypatch.setenv("LSG_DM_FORM", form)
    circuit = ls.parse(wl.brickwork(12, 12, seed=7, measure=False))
    noise = wl.dm_noise()
    got = ls.probabilities_array(circuit, noise, precision="c128")
    assert np.max(np.abs(got - cfg_arrays["cfg2_plain_probs"])) < ATOL_F64
    e = cfg["cfg2_plain_expectation"]
    assert abs(ls.expectation(circuit, e["label"], noise, precision="c128") - e["value"]) < ATOL_F64


def test_midcircuit_serial_counts_and_generator_match_orrery(cfg):
    """18 qubits x 16 rounds, 64 shots, seed 7, in Orrery's draw order (complex128)."""
    g = cfg["cfg3_serial64"]
    c = ls.parse(wl.midcircuit(*g["qasm_args"]))
    noise = NoiseModel.uniform(single=1e-3, two=1e-2)
    rng = np.random.default_rng(g["seed"])
    counts, report = trajectories.run_shots(c, g["shots"], noise, rng, _lib.C128, "serial")
    want: dict[int, int] = {}
    for bits in g["shot_bits"]:
        want[bits] = want.get(bits, 0) + 1
    assert counts == want, report
    state = rng.bit_generator.state["state"]
    assert (str(state["state"]), str(state["inc"])) == (g["rng_state"], g["rng_inc"])
    r = ls.run(c, shots=g["shots"], seed=g["seed"], noise=noise, method="trajectories")
    assert r.counts == g["counts"] and r.counts_digest == g["counts_digest"]


def _tableau(circuit) -> st.Tableau:
    enc = st.Encoder(None)
    t = st.Tableau(circuit.num_qubits)
    t.apply(enc.encode(all_gates(circuit.operations), False), enc)
    return t


def test_stabilizer_2048_qubits_1000_layers_bit_exact(cfg, cfg_arrays):
    """The benchmark's Clifford workload at full size: tableau, x0, row basis and counts."""
    g = cfg["cfg4_full"]
    n, layers, seed = g["qasm_args"]
    c = wl.clifford_layers_circuit(n, layers, seed=seed)
    assert c.digest() == g["circuit_digest"]
    t = _tableau(c)
    try:
        x, z, r = t.arrays()
        digest = hashlib.sha256(np.ascontiguousarray(x, dtype=np.uint8).tobytes() + np.ascontiguousarray(z, dtype=np.uint8).tobytes()
                                + np.ascontiguousarray(r, dtype=np.uint8).tobytes()).hexdigest()  # fmt: skip
        assert digest == g["tableau_sha256"]
        x0, basis = t.support(list(range(n)))
        assert np.array_equal(np.asarray(x0, dtype=np.uint8), cfg_arrays["cfg4_x0"])
        assert len(basis) == g["basis_rows"]
        assert hashlib.sha256(np.ascontiguousarray(basis, dtype=np.uint8).tobytes()).hexdigest() == g["basis_sha256"]
    finally:
        t.free()
    res = ls.run(c, shots=g["shots"], seed=g["seed"], noise=wl.stabilizer_noise(1e-3))
    assert res.method == g["method"]
    ones = np.zeros(n, dtype=np.int64)
    for key, count in res.counts.items():
        ones += count * (np.frombuffer(key.encode(), dtype=np.uint8)[::-1] == ord("1"))
    assert np.array_equal(ones, cfg_arrays["cfg4_ones"])
    assert len(res.counts) == g["distinct"] and res.counts_digest == g["counts_digest"]


def test_every_clifford_gate_on_the_device_tableau(cfg, cfg_arrays):
    """Every Clifford gate name Orrery knows (twice, shuffled) on a 6-qubit device tableau."""
    lines = ["OPENQASM 3.0;", 'include "stdgates.inc";', "qubit[6] q;"]
    for name, params, qs in cfg["clifford_maps"]["program"]:
        head = f"{name}({', '.join(repr(float(p)) for p in params)})" if params else name
        lines.append(f"{head} " + ", ".join(f"q[{q}]" for q in qs) + ";")
    c = ls.parse("\n".join(lines) + "\n")
    t = _tableau(c)
    try:
        x, z, r = t.arrays()
    finally:
        t.free()
    assert np.array_equal(x, cfg_arrays["cliff6_x"])
    assert np.array_equal(z, cfg_arrays["cliff6_z"])
    assert np.array_equal(r, cfg_arrays["cliff6_r"])
