"""The command-line front end driving the GPU engine, in the sequence of Orrery's CLI test
(``tests/test_sim.py:277-298``): run, run --json with noise, verify (match and mismatch), state
with amplitudes, expect, and a program error."""

from __future__ import annotations

import json

import pytest

from lucivant_sim_gb300.cli import main

pytestmark = pytest.mark.gpu

BELL = 'OPENQASM 3; include "stdgates.inc"; qubit[2] q; bit[2] c; h q[0]; cx q[0], q[1]; c = measure q;'


def test_cli_run_state_expect_verify(tmp_path, capsys):
    program = tmp_path / "bell.qasm"
    program.write_text(BELL)
    assert main(["run", str(program), "--shots", "200", "--seed", "3"]) == 0
    out = capsys.readouterr().out
    assert "fingerprint sha256:" in out and "2 qubits · 200 shots" in out
    assert main(["run", str(program), "--shots", "200", "--seed", "3", "--two", "0.02", "--json"]) == 0
    saved = tmp_path / "r.json"
    saved.write_text(capsys.readouterr().out)
    record = json.loads(saved.read_text())
    assert record["method"] == "density_matrix" and sum(record["counts"].values()) == 200
    assert main(["verify", str(saved), str(program), "--two", "0.02"]) == 0
    assert "verified" in capsys.readouterr().out
    assert main(["verify", str(saved), str(program)]) == 1
    assert "MISMATCH" in capsys.readouterr().out
    assert main(["state", str(program), "--amplitudes"]) == 0
    out = capsys.readouterr().out
    assert "+0.707107" in out and "|00>" in out and "|11>" in out
    assert main(["expect", str(program), "ZZ"]) == 0
    assert capsys.readouterr().out.strip() == "1"
    assert main(["expect", str(program), '{"ZI": 0.5, "XX": 1}']) == 0
    assert float(capsys.readouterr().out) == pytest.approx(1.0, abs=1e-12)
    bad = tmp_path / "bad.qasm"
    bad.write_text("OPENQASM 3; qubit q; nope q;")
    assert main(["run", str(bad)]) == 2
    assert "unknown gate 'nope'" in capsys.readouterr().err
