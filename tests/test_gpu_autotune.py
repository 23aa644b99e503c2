"""The autotuner on the GPU: every candidate plan gives the oracle's results within the engine's
tolerances, the fastest is kept and found again from the cache file."""

from __future__ import annotations

import json

import numpy as np
import pytest

import lucivant_sim_gb300 as ls
from lucivant_sim_gb300 import _lib, autotune, engine, workloads as wl
from lucivant_sim_gb300.batch import DensityBatch
from oracle import dense

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,tol", [("c128", 1e-12), ("c64", 1e-6)])
def test_every_candidate_matches_the_oracle_and_the_choice_is_cached(tmp_path, monkeypatch, precision, tol):
    monkeypatch.setenv("LSG_TUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setenv("LSG_JIT", "1")  # specialized passes: the CTAs-per-SM choice applies
    circuit = ls.parse(wl.brickwork(6, 4, seed=3, measure=False))
    noises = wl.dm_noise_instances(4, seed=2)
    want = np.stack([dense.probabilities_array(circuit, nm) for nm in noises])
    code = engine.REAL_OF[engine.precision_code(precision)]
    ops = engine.ptm_oplist(circuit, noises)
    with _lib.Register(12, code, batch=4) as reg:
        for opts in autotune.candidates(12, code):
            prog = _lib.Program(reg, ops, opts)
            try:
                assert prog.specialized
                prog.run_from_basis(reg, 0)
                got = reg.probabilities(6, member=-1)
            finally:
                prog.free()
            err = np.max(np.abs(got - want)) if precision == "c128" else np.max(0.5 * np.abs(got - want).sum(axis=1))
            assert err < tol, opts
    b = DensityBatch(circuit, noises, precision=precision, autotune=True)
    try:
        assert b.tune is not None and not b.tune["cached"] and len(b.tune["candidates"]) >= 2
        b.evolve()
        got = b.probabilities()
    finally:
        b.free()
    err = np.max(np.abs(got - want)) if precision == "c128" else np.max(0.5 * np.abs(got - want).sum(axis=1))
    assert err < tol
    saved = json.loads((tmp_path / "tune.json").read_text())
    assert len(saved) == 1 and next(iter(saved.values()))["opts"] == b.tune["opts"]
    autotune._memory.clear()  # a later process: the choice comes from the file
    again = DensityBatch(circuit, wl.dm_noise_instances(4, seed=9), precision=precision, autotune=True)
    try:
        assert again.tune["cached"] and again.tune["opts"] == b.tune["opts"]
    finally:
        again.free()


def test_bad_plan_options_are_refused():
    with _lib.Register(8, _lib.C64) as reg:
        ops = engine.sv_oplist(ls.parse(wl.brickwork(8, 2, seed=1, measure=False)))
        for bad in (_lib.PlanOpts(tile_bits=14), _lib.PlanOpts(tile_bits=-1), _lib.PlanOpts(ctas=9),
                    _lib.PlanOpts(max_ops=500), _lib.PlanOpts(tile_bits=6, low_bits=7)):  # fmt: skip
            with pytest.raises(ValueError):
                _lib.Program(reg, ops, bad)
        prog = _lib.Program(reg, ops, _lib.PlanOpts(tile_bits=8, max_ops=3))
        try:
            assert prog.passes >= len(ops) // 3
        finally:
            prog.free()
