"""Run-time specialized passes (LSG_JIT=1) against the interpreting pass kernel: the same planned
program, run both ways on the same register contents, gives the same numbers (both evaluate the
same operator sequence per group; only the compiled code differs: constant positions, two groups
per thread, renames folded into neighbouring blocks' addresses), for statevector and Pauli-transfer
density registers of every precision."""

from __future__ import annotations

import numpy as np
import pytest

from lucivant_sim_gb300 import _lib, engine
from lucivant_sim_gb300 import workloads as wl
from lucivant_sim_gb300.qasm import parse

pytestmark = pytest.mark.gpu

def _same(got, want, precision):
    """Specialized passes give the interpreter's numbers: bit for bit, except that double-float
    passes leave out zero terms, which keeps each value but not always its split into two words
    (a last-bit difference of the pair)."""
    if precision == _lib.RD:
        return float(np.max(np.abs(got - want))) < 1e-13
    return np.array_equal(got, want)


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
    assert np.array_equal(got, want), f"max difference {np.max(np.abs(got - want))}"


@pytest.mark.parametrize("precision", [_lib.R64, _lib.R32, _lib.RD])
@pytest.mark.parametrize("n", [5, 8, 11, 12])
def test_pauli_transfer_program(precision, n, monkeypatch):
    c = parse(wl.brickwork(n, 12 if n == 12 else 4, seed=n, measure=False))  # n=12: the benchmark's shape
    noises = wl.dm_noise_instances(3, seed=n)
    ops = engine.ptm_oplist(c, noises)
    rng = np.random.default_rng(n)
    start = rng.normal(size=(3, 1 << (2 * n)))
    want = _run(2 * n, precision, 3, ops, start, False, monkeypatch)
    got = _run(2 * n, precision, 3, ops, start, True, monkeypatch)
    assert _same(got, want, precision), f"max difference {np.max(np.abs(got - want))}"
    if precision == _lib.RD:  # and the FP64 register's numbers to the FP64 tolerance
        f64 = _run(2 * n, _lib.R64, 3, ops, start, True, monkeypatch)
        assert np.max(np.abs(got - f64)) < 1e-12


@pytest.mark.parametrize("variant", [{"LSG_FFMA2": "1"}, {"LSG_FFMA2": "0"}, {"LSG_JIT_SPILL": "0"}, {"LSG_JIT_SPILL": "1"}])
def test_benchmark_shape_code_variants(variant, monkeypatch):
    """The benchmark's circuit (12 qubits, 12 layers) as a real32 Pauli-transfer program: packed
    group pairs (fma.rn.f32x2) or not, passes that spill rebuilt for fewer CTAs per SM or not —
    every variant gives the interpreter's register bit for bit (defaults: packed, rebuilt)."""
    for k, v in variant.items():
        monkeypatch.setenv(k, v)
    c = parse(wl.brickwork(12, 12, seed=12, measure=False))
    ops = engine.ptm_oplist(c, wl.dm_noise_instances(2, seed=9))
    start = np.random.default_rng(9).normal(size=(2, 1 << 24))
    want = _run(24, _lib.R32, 2, ops, start, False, monkeypatch)
    got = _run(24, _lib.R32, 2, ops, start, True, monkeypatch)
    assert np.array_equal(got, want), f"max difference {np.max(np.abs(got - want))}"


def _from_basis_pair(nbits, precision, batch, ops, index, jit, monkeypatch):
    monkeypatch.setenv("LSG_JIT", "1" if jit else "0")
    with _lib.Register(nbits, precision, batch) as a, _lib.Register(nbits, precision, batch) as b:
        prog = _lib.Program(a, ops)
        try:
            a.set_basis(index)
            prog.run(a)
            prog.run_from_basis(b, index)
            assert prog.basis_bytes_per_run < prog.bytes_per_run  # the first passes skip zero tiles
            return a.download(), b.download()
        finally:
            prog.free()


@pytest.mark.parametrize("jit", [False, True])
@pytest.mark.parametrize("precision", [_lib.C128, _lib.C64])
def test_statevector_run_from_basis(precision, jit, monkeypatch):
    """Skipping tiles that are still zero gives exactly the full run's state, from |0..0> and from
    other basis states (their bits are the fixed values ORed into every tile's base)."""
    n = 16
    ops = engine.sv_oplist(parse(wl.brickwork(n, 3, seed=4, measure=False)))
    for index in (0, 0b1011_0000_0110_0101, (1 << n) - 1):
        want, got = _from_basis_pair(n, precision, 1, ops, index, jit, monkeypatch)
        assert np.array_equal(got, want), f"index {index}: max difference {np.max(np.abs(got - want))}"


@pytest.mark.parametrize("jit", [False, True])
@pytest.mark.parametrize("precision", [_lib.R64, _lib.R32, _lib.RD])
def test_pauli_transfer_run_from_basis(precision, jit, monkeypatch):
    n = 10
    c = parse(wl.brickwork(n, 6, seed=2, measure=False))
    ops = engine.ptm_oplist(c, wl.dm_noise_instances(2, seed=2))
    for index in (0, 0b10_0110_1001):
        want, got = _from_basis_pair(2 * n, precision, 2, ops, index, jit, monkeypatch)
        assert _same(got, want, precision), f"index {index}: max difference {np.max(np.abs(got - want))}"


def test_program_outlives_its_register(monkeypatch):
    """A program does not hold its creating register's stream: freeing the register first, then
    running the program on another register and freeing it, is well defined."""
    monkeypatch.setenv("LSG_JIT", "1")
    ops = engine.sv_oplist(parse(wl.brickwork(12, 2, seed=1, measure=False)))
    a = _lib.Register(12, _lib.C64)
    prog = _lib.Program(a, ops)
    a.free()
    with _lib.Register(12, _lib.C64) as b, _lib.Register(12, _lib.C64) as c:
        prog.run_from_basis(b, 0)
        c.set_basis(0)
        prog.run(c)
        assert np.array_equal(b.download(), c.download())
    prog.free()


@pytest.mark.parametrize("precision", [_lib.C128, _lib.C64])
def test_apply_from_basis_equals_set_basis_and_apply(precision):
    """The one-call evolution from a basis state (lsg_apply_from_basis) gives exactly the state of
    set_basis + lsg_apply, for a statevector and a complex vectorised density matrix."""
    sv_ops = engine.sv_oplist(parse(wl.brickwork(15, 3, seed=8, measure=False)))
    c = parse(wl.brickwork(6, 2, seed=8, measure=False))
    dm_ops = engine.dm_oplist(c, [wl.dm_noise()])
    for nbits, ops, index in ((15, sv_ops, 0), (15, sv_ops, 12345), (12, dm_ops, 0)):
        with _lib.Register(nbits, precision) as a, _lib.Register(nbits, precision) as b:
            a.set_basis(index)
            a.apply(ops)
            b.apply_from_basis(ops, index)
            assert np.array_equal(a.download(), b.download())


def test_module_cache_eviction(monkeypatch):
    """With room for two cached shapes, a third specialized program evicts the oldest; a program
    still alive keeps its own kernels, and programs of evicted shapes recompile correctly."""
    monkeypatch.setenv("LSG_JIT_CACHE_MAX", "2")
    monkeypatch.setenv("LSG_JIT", "1")
    rng = np.random.default_rng(7)
    start = rng.normal(size=(1, 1 << 10)) + 1j * rng.normal(size=(1, 1 << 10))
    opsets = [engine.sv_oplist(parse(wl.brickwork(10, 2, seed=40 + i, measure=False))) for i in range(4)]
    with _lib.Register(10, _lib.C64) as keep_reg:
        keep = _lib.Program(keep_reg, opsets[0])  # alive across the evictions
        assert keep.specialized
        for ops in opsets[1:] + opsets[:1]:
            _run(10, _lib.C64, 1, ops, start, True, monkeypatch)
        keep_reg.upload(start)
        keep.run(keep_reg)
        keep.run(keep_reg)  # twice, as _run does
        got = keep_reg.download()
        keep.free()
    want = _run(10, _lib.C64, 1, opsets[0], start, False, monkeypatch)
    assert np.array_equal(got, want)


def _random_ops(rng, nbits, real):
    """1- and 2-bit matrices, diagonals and permutations (some unit-phase: renames) on random bits."""
    ops = _lib.OpList()
    for _ in range(int(rng.integers(20, 90))):
        kind = int(rng.choice([_lib.OP_MATRIX, _lib.OP_DIAG, _lib.OP_PERM, _lib.OP_MATRIX]))
        k = int(rng.choice([1, 2, 2]))
        bits = [int(b) for b in rng.choice(nbits, size=k, replace=False)]
        d = 1 << k
        if kind == _lib.OP_MATRIX:
            m = np.linalg.qr(rng.normal(size=(d, d)) + (0 if real else 1j * rng.normal(size=(d, d))))[0]
            ops.add(kind, bits, np.asarray(m, dtype=complex))
        elif kind == _lib.OP_DIAG:
            ops.add(kind, bits, (rng.choice([-1.0, 1.0], size=d) if real else np.exp(1j * rng.uniform(0, 6.3, size=d))).astype(complex))
        else:
            phases = np.ones(d) if rng.random() < 0.5 else rng.choice([-1.0, 1.0], size=d)
            ops.add(kind, bits, np.concatenate([phases, rng.permutation(d)]).astype(complex))
    return ops


@pytest.mark.parametrize("precision", [_lib.C128, _lib.C64, _lib.R32, _lib.RD])
def test_random_programs(precision, monkeypatch):
    """Random programs (random bit positions: renames that fold or not, strided blocks, pairs,
    vector accesses) give the interpreter's register exactly when specialized."""
    rng = np.random.default_rng(100 + precision)
    real = precision in (_lib.R64, _lib.R32, _lib.RD)
    for nbits in (14, 16, 18):  # even: a Pauli-transfer register holds two bits per qubit
        ops = _random_ops(rng, nbits, real)
        start = rng.normal(size=(2, 1 << nbits))
        if not real:
            start = start + 1j * rng.normal(size=(2, 1 << nbits))
        want = _run(nbits, precision, 2, ops, start, False, monkeypatch)
        got = _run(nbits, precision, 2, ops, start, True, monkeypatch)
        assert _same(got, want, precision), f"{nbits} bits: max difference {np.max(np.abs(got - want))}"
