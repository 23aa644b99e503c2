"""Ragged runs: programs on registers of uneven widths and batches launched together, pass k of
every program in launch k (``lsg_programs_run_ragged``). Each register must hold exactly what its
program run alone leaves (same interpreter, same arithmetic: bit-identical)."""

from __future__ import annotations

import numpy as np
import pytest

from lucivant_sim_gb300 import _lib, engine, qasm, serve, workloads as wl
from lucivant_sim_gb300.noise import NoiseModel

pytestmark = pytest.mark.gpu


def _jobs(precision: int):
    """(register shape, operator list) of a statevector mix: widths 2..18, one 4-member sweep."""
    out = []
    for i, n in enumerate([2, 3, 5, 7, 8, 10, 11, 13, 14, 16, 18]):
        c = qasm.parse(wl.brickwork(n, 6 + i, seed=40 + i, measure=False))
        out.append(((n, precision, 1), engine.sv_oplist(c)))
    template = wl.hea_template(9, 2)
    rng = np.random.default_rng(3)
    params = [{f"p{k}": float(v) for k, v in enumerate(rng.uniform(0, 6.28, 36))} for _ in range(4)]
    out.append(((9, precision, 4), serve.sweep_oplist([qasm.parse(template, p) for p in params])))
    return out


def _alone(shape, ops, index):
    with _lib.Register(*shape) as reg:
        prog = _lib.Program(reg, ops)
        try:
            prog.run_from_basis(reg, index)
            reg.sync()
            return reg.download()
        finally:
            prog.free()


@pytest.mark.parametrize("precision", [_lib.C64, _lib.C128])
def test_ragged_statevectors_equal_each_run_alone(precision):
    jobs = _jobs(precision)
    rng = np.random.default_rng(7)
    index = [int(rng.integers(0, 1 << shape[0])) for shape, _ in jobs]
    regs = [_lib.Register(*shape) for shape, _ in jobs]
    progs = [_lib.Program(r, ops) for r, (_, ops) in zip(regs, jobs, strict=True)]
    try:
        ms = _lib.run_ragged(list(zip(progs, regs, strict=True)), index=index, timed=True)
        assert ms is not None and len(ms) == max(p.passes for p in progs) and np.all(ms > 0)
        got = [r.download() for r in regs]
        # a second ragged run on the same registers starts again from the basis states
        _lib.run_ragged(list(zip(progs, regs, strict=True)), index=index)
        again = [r.download() for r in regs]
    finally:
        for p in progs:
            p.free()
        for r in regs:
            r.free()
    for (shape, ops), g, a, i in zip(jobs, got, again, index, strict=True):
        want = _alone(shape, ops, i)
        assert np.array_equal(g, want), shape
        assert np.array_equal(a, want), shape
        assert np.allclose(np.sum(np.abs(g) ** 2, axis=1), 1.0, atol=1e-5)


def test_ragged_pauli_transfer_registers_with_noise():
    """Noisy density matrices of 2..6 qubits in real32 Pauli-transfer registers (4..12 bits)."""
    noise = NoiseModel.uniform(single=2e-3, two=1e-2)
    jobs = []
    for i, n in enumerate([2, 3, 4, 5, 6]):
        c = qasm.parse(wl.brickwork(n, 4 + i, seed=70 + i, measure=False))
        jobs.append(((2 * n, _lib.R32, 1), engine.ptm_oplist(c, [noise])))
    regs = [_lib.Register(*shape) for shape, _ in jobs]
    progs = [_lib.Program(r, ops) for r, (_, ops) in zip(regs, jobs, strict=True)]
    try:
        _lib.run_ragged(list(zip(progs, regs, strict=True)))
        got = [r.download() for r in regs]
    finally:
        for p in progs:
            p.free()
        for r in regs:
            r.free()
    for (shape, ops), g in zip(jobs, got, strict=True):
        want = _alone(shape, ops, 0)
        assert np.array_equal(g, want), shape
        assert abs(g[0, 0] - 1.0) < 1e-6  # trace preserved: the identity coefficient stays 1


def test_ragged_refuses_mixed_precisions_and_repeated_registers():
    c = qasm.parse(wl.brickwork(4, 3, seed=1, measure=False))
    ops = engine.sv_oplist(c)
    with _lib.Register(4, _lib.C64) as a, _lib.Register(4, _lib.C128) as b:
        pa, pb = _lib.Program(a, ops), _lib.Program(b, ops)
        try:
            with pytest.raises(ValueError, match="another precision"):
                _lib.run_ragged([(pa, a), (pb, b)])
            with pytest.raises(ValueError, match="appears twice"):
                _lib.run_ragged([(pa, a), (pa, a)])
            with _lib.Register(4, _lib.C64) as a2:
                with pytest.raises(ValueError, match="another basis index"):
                    _lib.run_ragged([(pa, a), (pa, a2)], index=[0, 3])
                _lib.run_ragged([(pa, a), (pa, a2)], index=[2, 2])  # one program, two registers
                assert np.array_equal(a.download(), a2.download())
        finally:
            pa.free()
            pb.free()
