"""Run-time specialized passes (LSG_JIT=1) against the interpreting pass kernel: the same planned
program, run both ways on the same register contents, agrees to rounding (both evaluate the same
operator sequence per group; only the compiled code differs), for statevector and Pauli-transfer
density registers of every precision."""

from __future__ import annotations

import numpy as np
import pytest

from lucivant_sim_gb300 import _lib, engine
from lucivant_sim_gb300 import workloads as wl
from lucivant_sim_gb300.qasm import parse

pytestmark = pytest.mark.gpu

TOL = {_lib.C128: 1e-12, _lib.C64: 2e-5, _lib.R64: 1e-12, _lib.R32: 2e-5}


def _run(reg_bits, precision, batch, ops, start, jit, monkeypatch):
    monkeypatch.setenv("LSG_JIT", "1" if jit else "0")
    with _lib.Register(reg_bits, precision, batch) as reg:
        reg.upload(start)
        prog = _lib.Program(reg, ops)
        try:
            assert prog.specialized == jit
            prog.run(reg)
            prog.run(reg)  # twice: the cached module and its launch state are reused
            return reg.download()
        finally:
            prog.free()


@pytest.mark.parametrize("precision", [_lib.C128, _lib.C64])
@pytest.mark.parametrize("n", [9, 14, 18])
def test_statevector_program(precision, n, monkeypatch):
    c = parse(wl.brickwork(n, 5, seed=n, measure=False))
    ops = engine.sv_oplist(c)
    rng = np.random.default_rng(n)
    start = rng.normal(size=(2, 1 << n)) + 1j * rng.normal(size=(2, 1 << n))
    start /= np.linalg.norm(start, axis=1, keepdims=True)
    want = _run(n, precision, 2, ops, start, False, monkeypatch)
    got = _run(n, precision, 2, ops, start, True, monkeypatch)
    assert np.max(np.abs(got - want)) < TOL[precision]


@pytest.mark.parametrize("precision", [_lib.R64, _lib.R32])
@pytest.mark.parametrize("n", [5, 8, 11])
def test_pauli_transfer_program(precision, n, monkeypatch):
    c = parse(wl.brickwork(n, 4, seed=n, measure=False))
    noises = wl.dm_noise_instances(3, seed=n)
    ops = engine.ptm_oplist(c, noises)
    rng = np.random.default_rng(n)
    start = rng.normal(size=(3, 1 << (2 * n)))
    want = _run(2 * n, precision, 3, ops, start, False, monkeypatch)
    got = _run(2 * n, precision, 3, ops, start, True, monkeypatch)
    scale = np.max(np.abs(want))
    assert np.max(np.abs(got - want)) < TOL[precision] * scale
