"""Whole-block fusion: a register block whose operators cost more than one dense 2^u x 2^u product
is replaced by that product, formed in FP64 on the host and rounded once. Fused and unfused
programs must agree (complex128 to 1e-13, complex64 to the register's rounding), and the fused
complex128 path must still match the oracle."""

from __future__ import annotations

import numpy as np
import pytest

from lucivant_sim_gb300 import _lib, engine, qasm, serve, workloads as wl
from oracle import dense

pytestmark = pytest.mark.gpu


def _run(shape, ops):
    with _lib.Register(*shape) as reg:
        prog = _lib.Program(reg, ops)
        try:
            info = prog.pass_info()
            prog.run_from_basis(reg, 0)
            reg.sync()
            return reg.download(), info
        finally:
            prog.free()


@pytest.mark.parametrize("precision,tol", [(_lib.C128, 1e-13), (_lib.C64, 2e-5)])
@pytest.mark.parametrize("n,depth,seed", [(6, 12, 1), (14, 30, 2), (18, 40, 3)])
def test_fused_blocks_equal_unfused(precision, tol, n, depth, seed, monkeypatch):
    c = qasm.parse(wl.brickwork(n, depth, seed=seed, measure=False))
    ops = engine.sv_oplist(c)
    fused, info_f = _run((n, precision, 1), ops)
    monkeypatch.setenv("LSG_FUSE_BLOCKS", "0")
    plain, info_p = _run((n, precision, 1), ops)
    assert np.max(np.abs(fused - plain)) < tol
    # fusion replaces operators, never passes or tiles: the same passes and bytes
    assert np.array_equal(info_f["bytes"], info_p["bytes"]) and np.array_equal(info_f["blocks"], info_p["blocks"])
    # and it did take blocks: the fused passes count other floating-point work per element
    assert not np.array_equal(info_f["flops_per_element"], info_p["flops_per_element"])


@pytest.mark.parametrize("precision,tol", [(_lib.C128, 1e-13), (_lib.C64, 2e-5)])
def test_fused_blocks_with_per_member_data(precision, tol, monkeypatch):
    """A parameter sweep: the fused product is formed per member."""
    template = wl.hea_template(10, 3)
    rng = np.random.default_rng(9)
    params = [{f"p{k}": float(v) for k, v in enumerate(rng.uniform(0, 6.28, 60))} for _ in range(5)]
    ops = serve.sweep_oplist([qasm.parse(template, p) for p in params])
    fused, _ = _run((10, precision, 5), ops)
    monkeypatch.setenv("LSG_FUSE_BLOCKS", "0")
    plain, _ = _run((10, precision, 5), ops)
    assert np.max(np.abs(fused - plain)) < tol
    assert not np.allclose(fused[0], fused[1])  # the members differ


def test_fused_complex128_matches_the_oracle():
    for n, depth, seed in [(7, 20, 11), (10, 25, 12)]:
        c = qasm.parse(wl.brickwork(n, depth, seed=seed, measure=False))
        got, _ = _run((n, _lib.C128, 1), engine.sv_oplist(c))
        want = dense.evolve_sv(c)
        assert np.max(np.abs(got[0] - want)) < 1e-12
