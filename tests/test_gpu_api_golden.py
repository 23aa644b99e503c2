"""The drop-in functions on the GPU against Orrery's own results on seeded random programs over every
gate name, several measurement layouts and noise models (``tests/golden/sim.*``, made by running
Orrery): the same method and counts for the same seed (unless a shot lies on a CDF boundary),
probabilities, outcome probabilities (readout included), expectations and final states within
1e-12, all through the engine's complex128 path; and for programs with mid-circuit measurement,
conditions and reset (trajectories) and random Clifford layers (the stabilizer engine), the same
method and counts."""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

import lucivant_sim_gb300 as ls
from lucivant_sim_gb300 import noise as ns

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
TOL = 1e-12


def _cases():
    sys.path.insert(0, str(GOLDEN))
    try:
        from recipes import build_model
    finally:
        sys.path.remove(str(GOLDEN))
    data = json.loads((GOLDEN / "sim.json").read_text())
    with np.load(GOLDEN / "sim.npz") as npz:
        arrays = {k: npz[k] for k in npz.files}
    out = []
    for case in data["cases"]:
        steps = data["noises"][case["noise"]]
        out.append((case, None if steps is None else build_model(ns, steps), arrays))
    return out


CASES = _cases()


@pytest.mark.parametrize("index", range(len(CASES)), ids=[c[0]["name"] for c in CASES])
def test_public_functions_match_orrery(index):
    case, noise, arrays = CASES[index]
    src, name = case["qasm"], case["name"]
    r = ls.run(src, shots=3000, seed=case["seed"], noise=noise)
    assert r.method == case["method"]
    assert r.counts == case["counts"] or r.report.get("near_boundary", 0) > 0
    assert r.circuit_digest == case["circuit_digest"] and r.noise_digest == case["fingerprint_noise"]
    probs = ls.probabilities(src, noise)
    assert set(probs) == set(case["probabilities"])
    assert max(abs(probs[k] - v) for k, v in case["probabilities"].items()) < TOL
    if case["outcome_probabilities"]:
        op = ls.outcome_probabilities(src, noise)
        assert set(op) == set(case["outcome_probabilities"])
        assert max(abs(op[k] - v) for k, v in case["outcome_probabilities"].items()) < TOL
    for obs, value in zip(case["observables"], case["expectations"], strict=True):
        assert abs(ls.expectation(src, obs, noise) - value) < TOL, obs
    if f"{name}::statevector" in arrays:
        assert np.max(np.abs(ls.statevector(src) - arrays[f"{name}::statevector"])) < TOL
    else:
        assert np.max(np.abs(ls.density_matrix(src, noise) - arrays[f"{name}::density_matrix"])) < TOL


RUN_CASES = json.loads((GOLDEN / "sim.json").read_text())["run_cases"]


@pytest.mark.parametrize("index", range(len(RUN_CASES)), ids=[c["name"] for c in RUN_CASES])
def test_runs_of_dynamic_and_clifford_programs_match_orrery(index):
    case = RUN_CASES[index]
    sys.path.insert(0, str(GOLDEN))
    try:
        from recipes import build_model
    finally:
        sys.path.remove(str(GOLDEN))
    steps = json.loads((GOLDEN / "sim.json").read_text())["noises"][case["noise"]]
    noise = None if steps is None else build_model(ns, steps)
    r = ls.run(case["qasm"], shots=case["shots"], seed=case["seed"], noise=noise)
    assert r.method == case["method"]
    assert r.circuit_digest == case["circuit_digest"] and r.noise_digest == case["fingerprint_noise"]
    near = r.report.get("near_threshold", 0) + r.report.get("near_boundary", 0)
    assert r.counts == case["counts"] or near > 0
