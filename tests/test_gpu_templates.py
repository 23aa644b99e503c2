"""Circuit templates: one planned program per template, new parameters through
``lsg_program_set_data`` and every run as one CUDA graph launch (``lsg_program_graph_run``). Each
run must equal a program built from scratch for the same parameters (bit-identical: the same
kernels on the same data)."""

from __future__ import annotations

import numpy as np
import pytest

from lucivant_sim_gb300 import _lib, engine, qasm, workloads as wl

pytestmark = pytest.mark.gpu


def _params(n: int, layers: int, seed: int) -> dict[str, float]:
    rng = np.random.default_rng(seed)
    return {f"p{k}": float(v) for k, v in enumerate(rng.uniform(0, 2 * np.pi, 2 * n * layers))}


def _fresh(n: int, precision: int, ops: _lib.OpList, index: int = 0) -> np.ndarray:
    with _lib.Register(n, precision) as reg:
        prog = _lib.Program(reg, ops)
        try:
            prog.run_from_basis(reg, index)
            reg.sync()
            return reg.download()
        finally:
            prog.free()


@pytest.mark.parametrize("precision", [_lib.C64, _lib.C128])
@pytest.mark.parametrize("n,layers", [(6, 2), (12, 4), (17, 3)])
def test_template_graph_with_new_parameters_equals_a_fresh_program(precision, n, layers):
    template = wl.hea_template(n, layers)
    sets = [_params(n, layers, s) for s in range(4)]
    ops = [engine.sv_oplist(qasm.parse(template, p)) for p in sets]
    with _lib.Register(n, precision) as reg:
        prog = _lib.Program(reg, ops[0])
        try:
            got = []
            for i, o in enumerate(ops):
                if i:
                    prog.set_data(reg, o)
                prog.graph_run(reg)  # the first call runs and captures, the others replay
                reg.sync()
                got.append(reg.download())
            # the same parameters again after others: the graph reads the data set last
            prog.set_data(reg, ops[1])
            prog.graph_run(reg)
            reg.sync()
            again = reg.download()
        finally:
            prog.free()
    for o, g in zip(ops, got, strict=True):
        assert np.array_equal(g, _fresh(n, precision, o))
    assert np.array_equal(again, got[1])
    assert not np.allclose(got[0], got[1])


def test_template_graph_follows_register_and_basis_index():
    n, layers = 9, 3
    ops = engine.sv_oplist(qasm.parse(wl.hea_template(n, layers), _params(n, layers, 7)))
    with _lib.Register(n, _lib.C64) as a, _lib.Register(n, _lib.C64) as b:
        prog = _lib.Program(a, ops)
        try:
            prog.graph_run(a, 0)
            prog.graph_run(a, 0)  # replay
            prog.graph_run(b, 5)  # another register and index: captured again
            a.sync()
            b.sync()
            ga, gb = a.download(), b.download()
        finally:
            prog.free()
    assert np.array_equal(ga, _fresh(n, _lib.C64, ops, 0))
    assert np.array_equal(gb, _fresh(n, _lib.C64, ops, 5))


def test_set_data_refuses_another_structure():
    n = 8
    a = engine.sv_oplist(qasm.parse(wl.hea_template(n, 2), _params(n, 2, 1)))
    b = engine.sv_oplist(qasm.parse(wl.brickwork(n, 5, seed=3, measure=False)))
    with _lib.Register(n, _lib.C64) as reg:
        prog = _lib.Program(reg, a)
        try:
            with pytest.raises(_lib.EngineError, match="plan differently"):
                prog.set_data(reg, b)
            prog.graph_run(reg)  # still the first template's data
            reg.sync()
            got = reg.download()
        finally:
            prog.free()
    assert np.array_equal(got, _fresh(n, _lib.C64, a))
