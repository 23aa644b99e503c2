"""Host-side pins against Orrery's results at the benchmarked sizes (``tests/golden/configs.*``,
made by ``tests/golden/make_golden_configs.py`` running Orrery 0.3.0 itself).

No device is used: these check that the benchmark builds the same noise models and circuits
Orrery ran, that the host's Clifford conjugation tables (the engine's) and the oracle's own
restatement of them are Orrery's for every gate name, and that the oracle reproduces Orrery's per-shot trajectory
draws on the 18-qubit, 16-round workload.
"""

from __future__ import annotations

import json
import math
from pathlib import Path

import numpy as np
import pytest

import lucivant_sim_gb300 as ls
from lucivant_sim_gb300 import workloads as wl
from lucivant_sim_gb300.clifford import clifford_map, kind_of
from lucivant_sim_gb300.gates import GATES
from lucivant_sim_gb300.noise import NoiseModel
from oracle import clifford as oracle_clifford
from oracle import dense, tableau

GOLDEN = Path(__file__).resolve().parent / "golden"


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


def test_benchmark_noise_models_are_the_ones_orrery_ran(cfg):
    """The benchmark's 256 instances (seed 7) carry Orrery's noise models, digest for digest."""
    noises = wl.dm_noise_instances(256, seed=7)
    members = [int(k[len("cfg2_inst"):]) for k in cfg if k.startswith("cfg2_inst")]
    assert members, "no batched-instance fixtures"
    for m in members:
        assert noises[m].digest() == cfg[f"cfg2_inst{m}"]["noise_digest"], m
    assert wl.dm_noise().digest() == cfg["cfg2_plain"]["noise_digest"]
    assert NoiseModel.uniform(single=1e-3, two=1e-2).digest() == cfg["cfg3_serial64"]["noise_digest"]
    assert wl.stabilizer_noise(1e-3).digest() == cfg["cfg4_full"]["noise_digest"]


def test_fixture_outputs_are_consistent(cfg, cfg_arrays):
    """Each density-matrix fixture is a probability distribution whose <Z_i> agree with it."""
    for name, case in cfg.items():
        if not name.startswith("cfg2_") or name.endswith("expectation"):
            continue
        p = cfg_arrays[f"{name}_probs"]
        assert p.shape == (4096,) and abs(p.sum() - 1) < 1e-12
        idx = np.arange(4096)
        z0 = float(np.sum(p * (1 - 2 * (idx & 1))))
        assert abs(z0 - case["z"][0]) < 1e-12


def test_clifford_tables_are_orreys_for_every_gate(cfg, cfg_arrays):
    """The host's conjugation table and named kind of every gate Orrery knows, at Clifford
    parameter values, equal Orrery's bit for bit (they drive the tableau kernels and the oracle)."""
    maps = cfg["clifford_maps"]["maps"]
    assert len(maps) >= 60
    for key, info in maps.items():
        m = np.asarray(GATES[info["name"]].build(*info["params"]), dtype=np.complex128)
        cmap = clifford_map(m)
        assert cmap is not None, key
        assert np.array_equal(cmap.bits, cfg_arrays[f"cmap_bits::{key}"]), key
        assert np.array_equal(cmap.sign, cfg_arrays[f"cmap_sign::{key}"]), key
        assert kind_of(cmap) == info["kind"], key


def test_oracle_clifford_tables_are_orreys_for_every_gate(cfg, cfg_arrays):
    """The oracle derives its tables on its own (the image Pauli read off the matrix, not
    projected on the Pauli basis); they too equal Orrery's, kind included."""
    maps = cfg["clifford_maps"]["maps"]
    for key, info in maps.items():
        m = np.asarray(GATES[info["name"]].build(*info["params"]), dtype=np.complex128)
        table = oracle_clifford.conjugation_table(m)
        assert table is not None, key
        assert np.array_equal(table.bits, cfg_arrays[f"cmap_bits::{key}"]), key
        assert np.array_equal(table.sign, cfg_arrays[f"cmap_sign::{key}"]), key
        assert oracle_clifford.kind_of(table) == info["kind"], key


def test_oracle_tableau_matches_orrery_over_every_clifford_gate(cfg, cfg_arrays):
    """A 6-qubit circuit over every Clifford gate name (twice, shuffled): the oracle's tableau is
    Orrery's."""
    c = ls.parse(clifford_program(cfg["clifford_maps"]["program"]))
    t = tableau.reference_tableau(c)
    assert np.array_equal(t.x, cfg_arrays["cliff6_x"])
    assert np.array_equal(t.z, cfg_arrays["cliff6_z"])
    assert np.array_equal(t.r, cfg_arrays["cliff6_r"])


def clifford_program(applied: list) -> str:
    """OpenQASM text of the fixture's gate list (parameters written exactly)."""
    lines = ["OPENQASM 3.0;", 'include "stdgates.inc";', "qubit[6] q;"]
    for name, params, qs in applied:
        head = f"{name}({', '.join(repr(float(p)) for p in params)})" if params else name
        lines.append(f"{head} " + ", ".join(f"q[{q}]" for q in qs) + ";")
    return "\n".join(lines) + "\n"


def test_oracle_serial_trajectories_follow_orreys_draws(cfg):
    """The first 12 shots of the 18-qubit, 16-round mid-circuit workload (uniform noise 1e-3 /
    1e-2, seed 7): the oracle's outcomes are Orrery's shot for shot."""
    g = cfg["cfg3_serial64"]
    c = ls.parse(wl.midcircuit(*g["qasm_args"]))
    noise = NoiseModel.uniform(single=1e-3, two=1e-2)
    rng = np.random.default_rng(g["seed"])
    got = [dense.trajectory(c, noise, rng) for _ in range(12)]
    assert got == g["shot_bits"][:12]


def test_orrery_timings_recorded(cfg):
    """The fixtures record how long Orrery took on this workload (the CPU reference)."""
    for m in (0, 1, 128, 255):
        assert cfg[f"cfg2_inst{m}"]["orrery_seconds"] > 0
    assert math.isfinite(cfg["cfg4_full"]["orrery_run_seconds"])


def test_method_choice_is_orreys_for_every_method_name():
    """``choose_method`` against Orrery's own answers (``tests/golden/methods.json``, made by
    running Orrery): every method name, including the accelerator names and an unknown one, over
    Clifford circuits below and at the stabilizer threshold, with a non-Clifford gate, a
    three-qubit gate, mid-circuit measurement and reset, circuits at and above the
    density-matrix limits, and noise models with no rules, Pauli channels, readout only and a
    non-Pauli channel: the same method, or the same exception class and message."""
    import sys

    from lucivant_sim_gb300 import noise as ns
    from lucivant_sim_gb300 import simulator

    sys.path.insert(0, str(GOLDEN))
    try:
        from recipes import noise_model
    finally:
        sys.path.remove(str(GOLDEN))
    data = json.loads((GOLDEN / "methods.json").read_text())
    circuits = {name: ls.parse(src) for name, src in data["programs"].items()}
    assert len(data["cases"]) >= 500
    for case in data["cases"]:
        nm = noise_model(case["noise"], ns)
        where = (case["program"], case["noise"], case["method"])
        try:
            got = {"method": simulator.choose_method(circuits[case["program"]], nm, case["method"])}
        except Exception as exc:  # noqa: BLE001 - compared with Orrery's record
            got = {"error": type(exc).__name__, "message": str(exc)}
        want = {k: case[k] for k in ("method", "error", "message") if k in case and k != "method" or
                (k == "method" and "error" not in case and k in case)}
        assert got == want, where


def test_qasm_reader_is_orreys_on_valid_and_malformed_programs():
    """The OpenQASM reader against Orrery's own reader (``tests/golden/qasm.json``, made by running
    Orrery): for programs covering the language (OpenQASM 2 and 3 declarations, every statement
    kind, gate definitions, modifiers, inputs, physical qubits, ranges, conditions, expressions,
    comments) the same circuit — digest, sizes, registers, inputs, operation kinds, whether it is
    dynamic, final measurements, operation counts and bit-string formatting; for
    malformed programs reaching each of Orrery's error messages the same exception class, message,
    line and column."""
    from lucivant_sim_gb300 import qasm

    kind_names = {"gate": "Gate", "measure": "Measure", "reset": "Reset", "barrier": "Barrier",
                  "if": "IfElse", "gphase": "GlobalPhase"}  # fmt: skip
    data = json.loads((GOLDEN / "qasm.json").read_text())
    assert len(data["programs"]) >= 80
    for rec in data["programs"]:
        try:
            c = qasm.parse(rec["source"], rec["params"])
        except Exception as exc:  # noqa: BLE001 - compared with Orrery's record
            got = {"error": {"class": type(exc).__name__, "message": str(exc), "line": getattr(exc, "line", None),
                             "column": getattr(exc, "column", None)}}  # fmt: skip
        else:
            got = {"circuit": {
                "digest": c.digest(),
                "num_qubits": c.num_qubits,
                "num_clbits": c.num_clbits,
                "qregs": [[r.name, r.offset, r.size] for r in c.qregs],
                "cregs": [[r.name, r.offset, r.size] for r in c.cregs],
                "inputs": dict(c.inputs),
                "kinds": [kind_names[op.kind] for op in c.operations],
                "is_dynamic": c.is_dynamic(),
                "final_measurements": [list(p) for p in c.final_measurements()],
                "count_ops": c.count_ops(),
                "format_bits": [c.format_bits(b) for b in (0, 1, 5, (1 << c.num_clbits) - 1)] if c.num_clbits else [],
            }}  # fmt: skip
        want = {k: rec[k] for k in ("circuit", "error") if k in rec}
        assert got == want, rec["name"]


def test_noise_models_are_orreys():
    """Noise models against Orrery's own (``tests/golden/noise.*``, made by running Orrery): every
    channel factory over several parameters gives the same Kraus operators and mixture branches
    (to 1e-15) and description; the factories refuse the same parameters with the same messages;
    models with overlapping rules resolve every (gate, qubits) query to the same channel, give the
    same readout errors, descriptions and digests; calibrations read into the same models."""
    import sys

    from lucivant_sim_gb300 import noise as ns

    sys.path.insert(0, str(GOLDEN))
    try:
        from recipes import build_channel, build_model
    finally:
        sys.path.remove(str(GOLDEN))
    data = json.loads((GOLDEN / "noise.json").read_text())
    with np.load(GOLDEN / "noise.npz") as arrays:
        for i, rec in enumerate(data["channels"]):
            ch = build_channel(ns, rec["recipe"])
            where = rec["recipe"]
            assert [ch.name, ch.num_qubits, ch.describe()] == [rec["name"], rec["num_qubits"], rec["describe"]], where
            assert bool(getattr(ch, "analytic_depolarizing", False)) == rec["analytic_depolarizing"], where
            kraus = np.stack([np.asarray(k, dtype=np.complex128) for k in ch.kraus])
            assert kraus.shape == arrays[f"ch{i}::kraus"].shape, where
            assert np.max(np.abs(kraus - arrays[f"ch{i}::kraus"])) <= 1e-15, where
            if rec["mixture"] is None:
                assert ch.mixture is None, where
            else:
                assert [float(p) for p, _m in ch.mixture] == rec["mixture"], where
                mats = np.stack([np.asarray(m, dtype=np.complex128) for _p, m in ch.mixture])
                assert np.array_equal(mats, arrays[f"ch{i}::mixture"]), where
    for rec in data["bad_channels"]:
        with pytest.raises(Exception) as info:
            build_channel(ns, rec["recipe"])
        assert {"class": type(info.value).__name__, "message": str(info.value)} == rec["error"], rec["recipe"]
    with pytest.raises(ValueError) as info:
        build_model(ns, [["gate", ["depolarizing", [0.1, 2]], None, [0]]])
    assert str(info.value) == data["bad_attach"]["message"]
    for name, rec in data["models"].items():
        m = build_model(ns, rec["steps"])
        assert m.describe() == rec["describe"] and m.digest() == rec["digest"], name
        assert (m.has_gate_errors(), m.is_empty()) == (rec["has_gate_errors"], rec["is_empty"]), name
        for (gate, qubits), want in zip(data["queries"], rec["gate_error"], strict=True):
            ch = m.gate_error(gate, tuple(qubits))
            assert (None if ch is None else ch.describe()) == want, (name, gate, qubits)
        for q, want in enumerate(rec["readout_error"]):
            e = m.readout_error(q)
            assert (None if e is None else [e.p01, e.p10]) == want, (name, q)
    for rec in data["calibrations"]:
        m = ns.NoiseModel.from_calibration(rec["calibration"])
        assert (m.describe(), m.digest(), m.source) == (rec["describe"], rec["digest"], rec["source"])


def test_gates_results_and_command_line_are_orreys(monkeypatch):
    """Orrery's public surface that needs no simulation (``tests/golden/api.*``, made by running
    Orrery): every gate's matrix at seeded parameters (to 1e-15), arity and canonical name; matrix
    powers; the ``Result`` record of synthetic results (fingerprint, counts digest, dictionary form,
    frequencies, most frequent outcome); and the command line's help, version and argument errors
    (output and exit code, at a fixed terminal width)."""
    import contextlib
    import io

    from lucivant_sim_gb300 import cli, gates
    from lucivant_sim_gb300.simulator import Result

    data = json.loads((GOLDEN / "api.json").read_text())
    with np.load(GOLDEN / "api.npz") as arrays:
        assert sorted(gates.GATES) == [g["name"] for g in data["gates"]]
        for g in data["gates"]:
            m = np.asarray(gates.gate_matrix(g["name"], tuple(g["params"])), dtype=np.complex128)
            assert np.max(np.abs(m - arrays[f"gate::{g['name']}"])) <= 1e-15, g["name"]
            assert gates.GATES[g["name"]].qubits == g["qubits"] and gates.canonical_name(g["name"]) == g["canonical"]
        for i, p in enumerate(data["powers"]):
            u = gates.gate_matrix(p["name"], tuple([0.7] * gates.GATES[p["name"]].params))
            assert np.max(np.abs(gates.matrix_power(u, p["k"]) - arrays[f"power::{i}"])) <= 1e-14, p
    for rec in data["results"]:
        r = Result(**rec["fields"])
        assert (r.fingerprint, r.counts_digest, r.frequencies(), r.most_frequent()) == (
            rec["fingerprint"], rec["counts_digest"], rec["frequencies"], rec["most_frequent"])
        assert json.loads(json.dumps(r.to_dict())) == rec["to_dict"]
    monkeypatch.setenv("COLUMNS", data["columns"])
    for rec in data["cli"]:
        out, err = io.StringIO(), io.StringIO()
        with contextlib.redirect_stdout(out), contextlib.redirect_stderr(err):
            try:
                code = cli.main(rec["argv"])
            except SystemExit as exc:
                code = exc.code
        assert (code, out.getvalue(), err.getvalue()) == (rec["code"], rec["stdout"], rec["stderr"]), rec["argv"]


def _sim_cases():
    import sys

    from lucivant_sim_gb300 import noise as ns

    sys.path.insert(0, str(GOLDEN))
    try:
        from recipes import build_model
    finally:
        sys.path.remove(str(GOLDEN))
    data = json.loads((GOLDEN / "sim.json").read_text())
    arrays = dict(np.load(GOLDEN / "sim.npz"))
    for case in data["cases"]:
        steps = data["noises"][case["noise"]]
        yield case, (None if steps is None else build_model(ns, steps)), arrays


def test_oracle_matches_orreys_public_functions_on_random_programs():
    """The oracle against Orrery's public functions on seeded random programs over every gate name
    and several measurement layouts (``tests/golden/sim.*``, made by running Orrery): identical
    counts for the same seed, probabilities and outcome probabilities (readout included),
    expectations and final states within 1e-12."""
    for case, nm, arrays in _sim_cases():
        c = ls.parse(case["qasm"])
        counts, method, _ = dense.run_counts(c, 3000, case["seed"], nm)
        assert (method, counts) == (case["method"], case["counts"]), case["name"]
        probs = dense.probabilities_array(c, nm)
        n = c.num_qubits
        want = case["probabilities"]
        got = {format(i, f"0{n}b"): float(p) for i, p in enumerate(probs) if p > 1e-12}
        assert set(got) == set(want), case["name"]
        assert max(abs(got[k] - want[k]) for k in want) < 1e-12, case["name"]
        if case["outcome_probabilities"]:
            op = dense.outcome_probabilities(c, nm)
            assert set(op) == set(case["outcome_probabilities"]), case["name"]
            assert max(abs(op[k] - v) for k, v in case["outcome_probabilities"].items()) < 1e-12, case["name"]
        for obs, value in zip(case["observables"], case["expectations"], strict=True):
            assert abs(dense.expectation(c, obs, nm) - value) < 1e-12, (case["name"], obs)
        if f"{case['name']}::statevector" in arrays:
            assert np.max(np.abs(dense.evolve_sv(c) - arrays[f"{case['name']}::statevector"])) < 1e-12
        else:
            rho = dense.evolve_dm(c, nm).reshape(1 << n, 1 << n)
            assert np.max(np.abs(rho - arrays[f"{case['name']}::density_matrix"])) < 1e-12


def test_oracle_matches_orreys_runs_of_dynamic_and_clifford_programs():
    """The oracle against Orrery's ``run`` on seeded random programs with mid-circuit measurement,
    conditions and reset (trajectories, Orrery's draw order) and on random Clifford layers over
    every Clifford gate name at 12 to 16 qubits (the stabilizer engine): the same method and
    identical counts for the same seed."""
    import sys

    from lucivant_sim_gb300 import noise as ns

    sys.path.insert(0, str(GOLDEN))
    try:
        from recipes import build_model
    finally:
        sys.path.remove(str(GOLDEN))
    data = json.loads((GOLDEN / "sim.json").read_text())
    assert len(data["run_cases"]) >= 6
    for case in data["run_cases"]:
        steps = data["noises"][case["noise"]]
        nm = None if steps is None else build_model(ns, steps)
        counts, method, _ = dense.run_counts(ls.parse(case["qasm"]), case["shots"], case["seed"], nm)
        assert (method, counts) == (case["method"], case["counts"]), case["name"]
