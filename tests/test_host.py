"""Host-side logic without a GPU: the C ABI loads and exports what include/lsg.h declares, and
the operator lists the host builds mean the same thing as Orrery's evolution (checked by a small
NumPy interpreter of the operator list against the oracle)."""

from __future__ import annotations

import re
from pathlib import Path

import numpy as np
import pytest

import lucivant_sim_gb300 as ls
from lucivant_sim_gb300 import _lib, engine, workloads as wl
from lucivant_sim_gb300.noise import NoiseModel, depolarizing, thermal_relaxation
from oracle import dense

ROOT = Path(__file__).resolve().parents[1]


def declared_functions() -> set[str]:
    names: set[str] = set()
    for header in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(lsg_\w+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol():
    lib = _lib.library()
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(_lib.SIGNATURES) <= declared_functions()
    assert lib.lsg_version() >= 1 and lib.lsg_max_bits() == 26


def run_oplist(ops: _lib.OpList, nbits: int, state: np.ndarray, member: int = 0) -> np.ndarray:
    """Reference interpreter of an operator list (what the device does, one operator at a time)."""
    table, pool = ops.packed()
    cpool = pool.view(np.complex128)
    v = state.astype(np.complex128).copy()
    for row in table:
        kind, k, bits = int(row["kind"]), int(row["nbits"]), [int(b) for b in row["bits"][: row["nbits"]]]
        at = int(row["data"]) + member * int(row["batch_stride"])
        if kind == _lib.OP_SCALE:
            v = v * cpool[at]
            continue
        if kind == _lib.OP_DEPOL:
            kq = k // 2
            v = dense.depolarizing_trace(v, nbits, cpool[at].real, bits[:kq], bits[kq:])
            continue
        d = 1 << k
        if kind == _lib.OP_MATRIX:
            m = cpool[at : at + d * d].reshape(d, d)
        elif kind == _lib.OP_DIAG:
            m = np.diag(cpool[at : at + d])
        else:
            ph = cpool[at : at + d]
            src = cpool[at + d : at + 2 * d].real.astype(int)
            m = np.zeros((d, d), dtype=np.complex128)
            m[np.arange(d), src] = ph
        v = dense.apply_bits(v, nbits, m, bits)
    return v


def test_statevector_oplist_means_the_circuit():
    c = ls.parse(wl.brickwork(6, 4, seed=3))
    v0 = np.zeros(64, dtype=np.complex128)
    v0[0] = 1
    got = run_oplist(engine.sv_oplist(c), 6, v0)
    assert np.max(np.abs(got - dense.evolve_sv(c))) < 1e-12


def test_density_oplist_means_the_circuit(golden):
    c = ls.parse(golden["dm_channels"]["qasm"])
    noise = (
        NoiseModel()
        .add_gate_error(ls.amplitude_damping(0.1), gates="h")
        .add_gate_error(ls.pauli_channel({"XY": 0.03, "ZZ": 0.02}), gates="cx")
        .add_gate_error(depolarizing(0.2, 2), gates="cz")
        .add_gate_error(thermal_relaxation(50, 40, 3.0), qubits=[2])
    )
    n = c.num_qubits
    rho0 = np.zeros(1 << (2 * n), dtype=np.complex128)
    rho0[0] = 1
    got = run_oplist(engine.dm_oplist(c, [noise]), 2 * n, rho0)
    assert np.max(np.abs(got - dense.evolve_dm(c, noise))) < 1e-12


def _ptm_density(ops: _lib.OpList, n: int) -> np.ndarray:
    """Run a Pauli-transfer operator list from |0><0| and convert to the density matrix."""
    r0 = np.zeros(1 << (2 * n), dtype=np.complex128)
    r0[: 1 << n] = 1  # Tr(P |0><0|) = 1 for the diagonal Paulis
    r = run_oplist(ops, 2 * n, r0)
    assert not np.any(r.imag)
    return run_oplist(engine.ptm_to_density_ops(n), 2 * n, r)


def test_pauli_transfer_oplist_means_the_circuit(golden):
    """The real Pauli-transfer operators evolve the same density matrix as Orrery (every channel
    kind of the golden case, resets, Clifford and non-Clifford two-qubit gates)."""
    c = ls.parse(golden["dm_channels"]["qasm"])
    noise = (
        NoiseModel()
        .add_gate_error(ls.amplitude_damping(0.1), gates="h")
        .add_gate_error(ls.pauli_channel({"XY": 0.03, "ZZ": 0.02}), gates="cx")
        .add_gate_error(depolarizing(0.2, 2), gates="cz")
        .add_gate_error(thermal_relaxation(50, 40, 3.0), qubits=[2])
    )
    assert engine.ptm_capable(c, [noise])
    got = _ptm_density(engine.ptm_oplist(c, [noise]), c.num_qubits)
    assert np.max(np.abs(got - dense.evolve_dm(c, noise).reshape(-1))) < 1e-12
    src = ("OPENQASM 3; include \"stdgates.inc\"; qubit[3] q; h q[0]; s q[1]; cx q[0], q[2]; cz q[1], q[2];"
           " swap q[0], q[1]; rzz(0.3) q[0], q[2]; cy q[2], q[0]; sx q[1]; t q[2]; reset q[1]; crx(0.4) q[1], q[0];"
           " ecr q[0], q[2];")
    c = ls.parse(src)
    for nm in (None, wl.dm_noise()):
        got = _ptm_density(engine.ptm_oplist(c, [nm]), 3)
        assert np.max(np.abs(got - dense.evolve_dm(c, nm).reshape(-1))) < 1e-12
    assert not engine.ptm_capable(ls.parse("OPENQASM 3; qubit[3] q; ccx q[0], q[1], q[2];"), [None])


def test_pauli_transfer_cx_is_renames_and_signs():
    """A noisy cx becomes bit renames (no arithmetic) plus one diagonal: signs and the
    depolarising factor; a noisy u3 one dense 4x4 real operator."""
    c = ls.parse("OPENQASM 3; include \"stdgates.inc\"; qubit[2] q; cx q[0], q[1]; u3(0.1, 0.2, 0.3) q[0];")
    ops = engine.ptm_oplist(c, [wl.dm_noise()])
    kinds = [row[0] for row in ops.rows]
    assert kinds.count(_lib.OP_PERM) >= 2 and kinds.count(_lib.OP_DIAG) == 1 and kinds[-1] == _lib.OP_MATRIX
    assert all(row[1] == 2 for row in ops.rows if row[0] == _lib.OP_PERM)


def test_gf2_linear_permutations_decompose_into_renames():
    rng = np.random.default_rng(1)
    for nb in (2, 3, 4):
        for _ in range(20):
            while True:
                m = rng.integers(0, 2, size=(nb, nb))
                if round(abs(np.linalg.det(m))) % 2 == 1:
                    break
            def apply(mat, r):
                v = np.array([(r >> (nb - 1 - p)) & 1 for p in range(nb)])
                w = mat.dot(v) % 2
                return int(sum(int(b) << (nb - 1 - p) for p, b in enumerate(w)))
            src = np.array([apply(m, r) for r in range(1 << nb)])
            steps = engine._renames(src, nb)
            cur = np.arange(1 << nb)  # out[r] = in[cur[r]] after the steps so far
            for kind, a, b in steps:
                def one(r, kind=kind, a=a, b=b):
                    ba, bb = (r >> (nb - 1 - a)) & 1, (r >> (nb - 1 - b)) & 1
                    if kind == "cx":
                        return r ^ (ba << (nb - 1 - b))
                    return r ^ ((ba ^ bb) << (nb - 1 - a)) ^ ((ba ^ bb) << (nb - 1 - b))
                cur = np.array([cur[one(r)] for r in range(1 << nb)])
            assert np.array_equal(cur, src)
    assert engine._renames(np.array([1, 0, 2, 3]), 2) is None  # moves 0: not linear
    assert engine._renames(np.array([0, 1, 2, 4, 3, 5, 6, 7]), 3) is None


def test_matrix_classes():
    from lucivant_sim_gb300.gates import GATES

    kind, data = engine.classify(GATES["cx"].build())
    assert kind == _lib.OP_PERM and list(data[4:].real) == [0, 1, 3, 2]
    assert engine.classify(GATES["rz"].build(0.3))[0] == _lib.OP_DIAG
    assert engine.classify(GATES["h"].build())[0] == _lib.OP_MATRIX


def test_superoperators_are_trace_preserving():
    for ch in (thermal_relaxation(120, 90, 0.05), ls.amplitude_damping(0.3), depolarizing(0.1)):
        s = engine.superop(ch.kraus)
        # trace of the output = trace of the input for every input
        for r in range(4):
            e = np.zeros(4)
            e[r] = 1
            out = (s @ e).reshape(2, 2)
            assert abs(np.trace(out) - np.trace(e.reshape(2, 2))) < 1e-12
    s = engine.depolarizing_superop(0.2, 1)
    assert np.allclose(s, engine.superop(depolarizing(0.2).kraus), atol=1e-12)


def test_count_bits_packs_like_orrery():
    c = ls.parse("OPENQASM 3; qubit[3] q; bit[2] a; bit[1] b; a[1] = measure q[0]; b[0] = measure q[2];")
    bits = np.array([[1, 0], [1, 1], [0, 0], [1, 1]], dtype=np.uint8)
    from lucivant_sim_gb300.simulator import count_bits

    assert count_bits(c, bits, [1, 2]) == {"0 00": 1, "0 10": 1, "1 10": 2}
    # ordered by outcome string, also where numeric order is not string order (registers
    # declared out of clbit order)
    c2 = ls.parse("OPENQASM 3; qubit[4] q; bit[2] a; bit[2] b; a[0] = measure q[0]; a[1] = measure q[1]; "
                  "b[0] = measure q[2]; b[1] = measure q[3];")
    rng = np.random.default_rng(3)
    many = rng.integers(0, 2, (300, 4)).astype(np.uint8)
    for clbits in ([0, 1, 2, 3], [3, 1, 0, 2]):
        got = count_bits(c2, many, clbits)
        assert list(got) == sorted(got) and sum(got.values()) == 300


def test_pauli_masks():
    assert engine.pauli_masks("XYZI") == (0b1100, 0b0110)


def test_no_oracle_in_product():
    """The product never imports the oracle (it is test infrastructure only)."""
    for path in (ROOT / "lucivant_sim_gb300").rglob("*.py"):
        text = path.read_text()
        assert "import oracle" not in text and "from oracle" not in text, path


def test_library_pcg64_matches_numpy():
    """The engine's PCG64 (host build of the device code) regenerates NumPy's stream."""
    from lucivant_sim_gb300 import stabilizer as st

    for seed in (0, 7, 11, 2**40 + 3):
        rng = np.random.default_rng(seed)
        probe = np.random.default_rng(seed)
        raw = probe.bit_generator.random_raw(2000)
        for i in (0, 1, 2, 17, 999, 1999):
            assert st.pcg_raw(rng, i) == int(raw[i])


def test_uint8_integers_stream_layout():
    """integers(0, 2, uint8) is the top bit of each byte of the buffered uint32 stream."""
    rng = np.random.default_rng(3)
    vals = rng.integers(0, 2, size=37, dtype=np.uint8)
    raw = np.random.default_rng(3).bit_generator.random_raw(5)
    words = []
    for r in raw:
        words += [int(r) & 0xFFFFFFFF, int(r) >> 32]
    bytes_ = [(w >> (8 * i)) & 0xFF for w in words for i in range(4)]
    assert list(vals) == [b >> 7 for b in bytes_[:37]]


@pytest.mark.parametrize("tile,low", [(None, None), ("7", "3"), ("8", "3"), ("5", "2"), ("12", "6")])
def test_plans_are_well_formed(monkeypatch, tile, low):
    """The host planner's passes and register blocks are checked (lsg_plan validates them) for
    every shape the GPU tests force, for statevector, density and wide-gate operator lists."""
    if tile:
        monkeypatch.setenv("LSG_TILE_BITS", tile)
        monkeypatch.setenv("LSG_LOW_BITS", low)
    cases = [
        (engine.sv_oplist(ls.parse(wl.brickwork(9, 4, seed=1))), 9),
        (engine.dm_oplist(ls.parse(wl.brickwork(4, 3, seed=2, measure=False)), [wl.dm_noise()]), 8),
        (engine.dm_oplist(ls.parse(wl.brickwork(5, 2, seed=3, measure=False)),
                          [NoiseModel().add_gate_error(ls.pauli_channel({"XY": 0.1}), gates="cx")]), 10),
        (engine.sv_oplist(ls.parse("OPENQASM 3; qubit[6] q; h q; ccx q[0], q[3], q[5]; c4x q[5], q[1], q[2], q[0], q[4]; "
                                   "rz(0.3) q[2]; gphase(0.2); rzz(0.4) q[1], q[4];")), 6),
    ]
    cases.append((engine.ptm_oplist(ls.parse(wl.brickwork(4, 3, seed=2, measure=False)), [wl.dm_noise()]), 8))
    for ops, nbits in cases:
        for precision in (_lib.C128, _lib.C64, _lib.R64, _lib.R32):
            try:
                assert _lib.plan_passes(nbits, precision, ops) >= 1
            except ValueError as exc:  # a tile too small for a wide operator is refused, never malformed
                assert "does not fit" in str(exc), exc


def test_served_jobs_prepare_to_their_circuits():
    """A served parameter sweep is one batched operator list whose member b is parameter set b;
    sampled and noisy jobs carry the same operator lists as the direct API."""
    from lucivant_sim_gb300 import serve

    jobs = wl.served_mix(40, seed=11, widths=(3, 6), depths=(2, 12), sweep=3)
    kinds = {j["kind"] for j in jobs}
    assert kinds == {"expect", "density", "sample"}
    for job in jobs:
        prep = serve.prepare(job)
        if job["kind"] == "expect":
            sweep = serve.sweep_oplist([ls.parse(job["qasm"], p) for p in job["params"]])
            n = prep["nbits"]
            v0 = np.zeros(1 << n, dtype=np.complex128)
            v0[0] = 1
            for b, params in enumerate(job["params"]):
                want = dense.evolve_sv(ls.parse(job["qasm"], params))
                got = run_oplist(sweep, n, v0, member=b)
                assert abs(abs(np.vdot(want, got)) - 1) < 1e-12
            assert prep["batch"] == len(job["params"]) and len(prep["xmask"]) == 20
        else:
            c = ls.parse(job["qasm"])
            want = engine.sv_oplist(c) if job["kind"] == "sample" else engine.ptm_oplist(
                c, [NoiseModel.uniform(**serve.DEFAULT_NOISE)])
            assert prep.get("real", False) == (job["kind"] == "density")
            t0, p0 = want.packed()
            t1, p1 = prep["ops"]
            assert np.array_equal(t0, t1) and np.array_equal(p0, p1)


def test_deep_circuits_split_into_bounded_passes():
    """A pass holds at most 192 operators (their descriptors sit in shared memory beside the tile),
    so a deep circuit on few qubits plans into several passes instead of one oversized one."""
    ops = engine.sv_oplist(ls.parse(wl.brickwork(10, 120, seed=4)))
    assert len(ops) > 192 * 3
    for precision in (_lib.C128, _lib.C64):
        assert _lib.plan_passes(10, precision, ops) >= -(-len(ops) // 192)


def test_specialized_pass_source_compiles():
    """The run-time specializer's source for a Pauli-transfer program (two groups per thread,
    trace-preserving 4x4 operators, renames, diagonals) and a statevector program compiles with
    NVRTC for sm_103a; wide operators leave a program to the interpreter."""
    pytest.importorskip("ctypes")
    from lucivant_sim_gb300 import _lib, engine
    from lucivant_sim_gb300 import workloads as wl
    from lucivant_sim_gb300.qasm import parse

    c = parse(wl.brickwork(7, 2, seed=3, measure=False))
    ptm = engine.ptm_oplist(c, wl.dm_noise_instances(2, seed=3))
    src = _lib.specialized_source(14, _lib.R32, 2, ptm, compile=True)
    unpacked = "rb_tpd2<float" in src and "ld_split<float>" in src
    packed = "rp_tpd2<" in src and "ld_f2(" in src  # the default; unpacked with LSG_FFMA2=0
    assert (unpacked or packed) and "lsg_pass_0" in src
    sv = engine.sv_oplist(parse(wl.brickwork(14, 2, seed=3, measure=False)))
    src = _lib.specialized_source(14, _lib.C64, 1, sv, compile=True)
    assert "lsg::Cx<float>" in src
    wide = _lib.OpList()
    wide.add(_lib.OP_MATRIX, [0, 1, 2, 3, 4], np.eye(32, dtype=complex))
    assert _lib.specialized_source(14, _lib.C64, 1, wide) == ""


def test_packed_pair_source_compiles(monkeypatch):
    """Real32 group pairs are generated as packed 64-bit operands (fma.rn.f32x2), or unpacked with
    LSG_FFMA2=0; both compile and load the same addresses."""
    from lucivant_sim_gb300.qasm import parse

    c = parse(wl.brickwork(7, 3, seed=4, measure=False))
    ptm = engine.ptm_oplist(c, wl.dm_noise_instances(2, seed=5))
    monkeypatch.setenv("LSG_FFMA2", "0")
    plain = _lib.specialized_source(14, _lib.R32, 2, ptm)
    monkeypatch.setenv("LSG_FFMA2", "1")
    packed = _lib.specialized_source(14, _lib.R32, 2, ptm, compile=True)
    assert "rp_tpd2<" in packed and "ld_f2(" in packed and "ld_split<" not in packed
    assert "ld_split<float>" in plain and "rp_" not in plain
    addr = re.compile(r"tile \+ \(([^)]*)\)")
    assert sorted(addr.findall(plain)) == sorted(addr.findall(packed))
    # complex registers are never packed
    sv = engine.sv_oplist(parse(wl.brickwork(14, 2, seed=3, measure=False)))
    assert "rp_" not in _lib.specialized_source(14, _lib.C64, 1, sv)


def test_fused_blocks_and_lane_bits_in_specialized_source(monkeypatch):
    """Whole-block fusion gives complex programs dense block operators (rb_denseb), never real
    ones; the lane-bit choice moves group-index bits in some real32 blocks; both compile."""
    from lucivant_sim_gb300.qasm import parse

    sv = engine.sv_oplist(parse(wl.brickwork(14, 12, seed=5, measure=False)))
    fused = _lib.specialized_source(14, _lib.C64, 1, sv, compile=True)
    assert "rb_denseb<lsg::Cx<float>" in fused
    monkeypatch.setenv("LSG_FUSE_BLOCKS", "0")
    assert "rb_denseb" not in _lib.specialized_source(14, _lib.C64, 1, sv)
    monkeypatch.delenv("LSG_FUSE_BLOCKS")
    c = parse(wl.brickwork(12, 12, seed=7, measure=False))
    ptm = engine.ptm_oplist(c, wl.dm_noise_instances(2, seed=7))
    chosen = _lib.specialized_source(24, _lib.R32, 2, ptm, compile=True)
    assert "rb_denseb" not in chosen
    moved = re.compile(r"const uint32_t G = \(+uint32_t\(g\) >>")
    assert moved.search(chosen)
    monkeypatch.setenv("LSG_LANE_BITS", "0")
    plain = _lib.specialized_source(24, _lib.R32, 2, ptm)
    assert not moved.search(plain)
    # the same arithmetic: only the group enumeration differs
    calls = re.compile(r"r[bp]_\w+<[^>]*>\([^;]*;")
    assert calls.findall(plain) == calls.findall(chosen)


def test_new_entry_points_refuse_bad_arguments_before_any_device_call():
    lib = _lib.library()
    assert lib.lsg_programs_run_ragged(0, None, None, None, None) == _lib.LSG_E_ARG
    assert lib.lsg_program_set_data(None, None, None, 0, None, 0) == _lib.LSG_E_ARG
    assert lib.lsg_program_graph_run(None, None, 0) == _lib.LSG_E_ARG
    assert b"null" in lib.lsg_last_error() or b"bad" in lib.lsg_last_error()


def test_format_bits_many_matches_format_bits():
    from lucivant_sim_gb300.circuit import format_bits, format_bits_many

    rng = np.random.default_rng(5)
    for src in (
        'OPENQASM 3; qubit[5] q; bit[5] c;',
        'OPENQASM 3; qubit[6] q; bit[2] a; bit[3] b; bit[1] d;',
        'OPENQASM 2.0; qreg q[4]; creg c[4];',
    ):
        c = ls.parse(src)
        values = np.unique(rng.integers(0, 1 << c.num_clbits, size=40))
        assert format_bits_many(c, values) == [format_bits(c, int(v)) for v in values]
        assert format_bits_many(c, np.array([], dtype=np.int64)) == []


def test_pauli_transfer_oplist_batched_members():
    """A batched Pauli-transfer operator list (one channel stack per gate signature, equal gates
    classified once) gives every member its own noise model's density matrix."""
    c = ls.parse(wl.brickwork(3, 3, seed=4, measure=False))
    noises = wl.dm_noise_instances(3, seed=9)
    ops = engine.ptm_oplist(c, noises)
    assert any(row[4] for row in ops.rows)  # per-member data present
    n = c.num_qubits
    for m, nm in enumerate(noises):
        r = np.zeros(1 << (2 * n))
        r[: 1 << n] = 1.0  # |0..0><0..0|: every diagonal Pauli has coefficient 1
        r = run_oplist(ops, 2 * n, r, member=m).real
        got = run_oplist(engine.ptm_to_density_ops(n), 2 * n, r)
        assert np.max(np.abs(got - dense.evolve_dm(c, nm).reshape(-1))) < 1e-12, m


def test_planner_and_specializer_on_random_operator_lists():
    """Random operator lists (1-5 bit matrices, diagonals, permutations, global phases) on registers
    of 3-22 bits plan without an internal error in every precision (the planner checks every block's
    deposit masks and vector alignment), and the specializer writes their passes (or leaves a
    program with wide operators to the interpreter) for one and many starting tiles."""
    import os

    rng = np.random.default_rng(12)
    written = 0
    for trial in range(60):
        nbits = int(rng.choice([3, 8, 14, 20, 22]))
        wide = trial % 4 == 0  # a quarter of the programs may hold wider operators
        ops = _lib.OpList()
        for _ in range(int(rng.integers(1, 120))):
            kind = int(rng.choice([_lib.OP_MATRIX, _lib.OP_DIAG, _lib.OP_PERM, _lib.OP_MATRIX]))
            # register blocks take 1- and 2-bit operators (and diagonals); 3-5 bit matrices and
            # permutations run on the shared-memory path, which keeps a program interpreted
            k = int(rng.choice([1, 1, 2, 2, 2])) if not wide or rng.random() > 0.05 else int(rng.integers(3, 6))
            k = min(k, nbits)
            bits = [int(b) for b in rng.choice(nbits, size=k, replace=False)]
            d = 1 << k
            if kind == _lib.OP_MATRIX:
                ops.add(kind, bits, np.linalg.qr(rng.normal(size=(d, d)))[0].astype(complex))
            elif kind == _lib.OP_DIAG:  # real data: the real (Pauli-transfer) precisions take it too
                ops.add(kind, bits, rng.choice([-1.0, 0.5, 2.0], size=d).astype(complex))
            else:
                src = rng.permutation(d)
                ops.add(kind, bits, np.concatenate([np.ones(d), src]).astype(complex))
        for seeds in ("1", "64"):
            os.environ["LSG_PLAN_SEEDS"] = seeds
            try:
                for prec in (_lib.C128, _lib.C64, _lib.R64, _lib.R32):
                    assert _lib.plan_passes(nbits, prec, ops) >= 1
                    src = _lib.specialized_source(nbits, prec, 2, ops)
                    assert src == "" or "lsg_pass_0" in src
                    written += bool(src)
            finally:
                os.environ.pop("LSG_PLAN_SEEDS", None)
    assert written > 150  # the programs without operators wider than a register block


def test_gate_errors_over_many_models_match_each_model():
    """The batched rule lookup picks, for every model, the channel the model's own gate_error
    picks: specific rules beat general ones, later rules win ties, shapes may differ per model."""
    from lucivant_sim_gb300.noise import GateErrors

    rng = np.random.default_rng(5)
    models: list[NoiseModel | None] = []
    for i in range(40):
        if i % 13 == 7:
            models.append(None)
            continue
        m = NoiseModel()
        m.add_gate_error(depolarizing(float(rng.uniform(0, 0.1)), 1))
        m.add_gate_error(depolarizing(float(rng.uniform(0, 0.1)), 2))
        if i % 3 == 0:
            m.add_gate_error(depolarizing(float(rng.uniform(0, 0.1)), 1), gates="h")
        if i % 4 == 1:
            m.add_gate_error(depolarizing(float(rng.uniform(0, 0.1)), 1), qubits=[2])
            m.add_gate_error(depolarizing(float(rng.uniform(0, 0.1)), 2), gates=["cx"], qubits=[1, 0])
        if i % 5 == 2:
            m.add_gate_error(thermal_relaxation(50.0, 40.0, 0.1), gates=["x", "h"], qubits=[2])
        models.append(m)
    lookup = GateErrors(models)
    for name, qubits in [("h", (0,)), ("h", (2,)), ("x", (2,)), ("rz", (1,)), ("cx", (0, 1)), ("cx", (1, 2)),
                         ("u3", (2,)), ("cz", (1, 0)), ("ccx", (0, 1, 2))]:
        want = [None if m is None else m.gate_error(name, qubits) for m in models]
        got = lookup(name, qubits)
        assert all(a is b for a, b in zip(got, want)), (name, qubits)


def test_cli_arguments_and_errors_without_a_device(tmp_path, capsys):
    """The command-line front end: version, argument errors and program errors are reported
    before any device work, with Orrery's exit codes and wording."""
    from lucivant_sim_gb300 import cli

    with pytest.raises(SystemExit) as stop:
        cli.main(["--version"])
    assert stop.value.code == 0 and capsys.readouterr().out.startswith("lucivant-sim 0.3.0")
    bad = tmp_path / "bad.qasm"
    bad.write_text("OPENQASM 3; qubit q; nope q;")
    assert cli.main(["run", str(bad)]) == 2
    assert "unknown gate 'nope'" in capsys.readouterr().err
    assert cli.main(["state", str(tmp_path / "missing.qasm")]) == 2
    assert capsys.readouterr().err.startswith("lucivant-sim: ")
    with pytest.raises(SystemExit) as stop:
        cli.main(["run", str(bad), "--param", "theta"])
    assert "--param needs name=value" in str(stop.value.code)
    with pytest.raises(SystemExit):
        cli.main(["run", str(bad), "--method", "no_such_method"])
    capsys.readouterr()
    args = cli.build_parser().parse_args(["run", "x.qasm", "--two", "0.02"])
    nm = cli.noise_of(args)
    assert nm is not None and nm.gate_error("cx", (0, 1)) is not None and nm.gate_error("h", (0,)) is None
    assert cli.noise_of(cli.build_parser().parse_args(["run", "x.qasm"])) is None
    assert cli.parse_params(["a=0.5", " b =2"]) == {"a": 0.5, "b": 2.0}
    assert cli.bar(0.5) == "█" * 16 and cli.bar(0.0) == ""


def test_canonical_text_is_the_sorted_compact_json_of_the_canonical_form():
    """The digest's text, assembled from cached per-matrix texts, is character for character
    ``json.dumps(canonical, separators=(",", ":"), sort_keys=True)`` (the form Orrery hashes)."""
    import json

    sources = [
        wl.brickwork(12, 6, seed=7),
        wl.brickwork(6, 2, seed=3, measure=False),
        wl.midcircuit(8, 3, seed=5),
        'OPENQASM 3; include "stdgates.inc"; qubit[3] q; bit[2] a; bit[1] b; h q[0]; barrier q; gphase(0.3); '
        "a[0] = measure q[0]; if (a[0] == 1) { x q[1]; } else { z q[2]; } reset q[0]; b[0] = measure q[2];",
        'OPENQASM 2.0; include "qelib1.inc"; qreg q[2]; creg c[2]; u3(0.1,0.2,0.3) q[0]; cx q[0],q[1]; measure q -> c;',
        "OPENQASM 3; qubit[2] q; bit[2] c; U(0.5, -0.0, 1e-13) q[0]; c = measure q;",
    ]
    circuits = [ls.parse(s) for s in sources] + [wl.clifford_layers_circuit(16, 2, seed=3)]
    for c in circuits:
        assert c.canonical_text() == json.dumps(c.canonical(), separators=(",", ":"), sort_keys=True)


def test_density_batch_halves_decision(monkeypatch):
    """run_density_batch's halves, with a stand-in for the device batch: an even batch runs as two
    halves in member order unless a half would lose the specialization the whole batch gets."""
    from lucivant_sim_gb300 import batch as batch_mod

    made: list[list[int]] = []

    class FakeProgram:
        def __init__(self, n, specialized):
            self.specialized = specialized
            self.bytes_per_run = 100 * n

    class FakeBatch:
        specialize_from = 4  # members from which the stand-in policy specializes

        def __init__(self, circuit, noises, precision, autotune=None):
            made.append(list(noises))
            self.members = list(noises)
            self.program = FakeProgram(len(noises), len(noises) >= self.specialize_from)

        def evolve(self):
            pass

        def probabilities(self):
            return np.array([[m, m] for m in self.members], dtype=float)

        def expectations(self, labels):
            return np.array([self.members for _ in labels], dtype=float)

        def free(self):
            pass

    monkeypatch.setattr(batch_mod, "DensityBatch", FakeBatch)
    monkeypatch.setattr(_lib, "jit_wanted", lambda nbytes: nbytes >= 400)
    assert batch_mod.halves([1, 2, 3]) == [[1, 2, 3]] and batch_mod.halves([]) == [[]]
    assert batch_mod.halves([1, 2, 3, 4], split=False) == [[1, 2, 3, 4]]
    for members, split, want in [
        (list(range(8)), True, [[0, 1, 2, 3], [4, 5, 6, 7]]),  # halves stay specialized
        (list(range(4)), True, [[0, 1], [0, 1, 2, 3]]),  # a half would not be: the whole batch
        (list(range(2)), True, [[0], [1]]),  # neither would be: halves
        (list(range(5)), True, [[0, 1, 2, 3, 4]]),  # odd: one batch
        (list(range(8)), False, [[0, 1, 2, 3, 4, 5, 6, 7]]),
    ]:
        made.clear()
        probs, exps = batch_mod.run_density_batch(None, members, ["Z", "ZZ"], split=split)
        assert made == want
        assert probs[:, 0].tolist() == members and exps.shape == (2, len(members))
        assert exps[0].tolist() == members


def test_public_header_is_plain_c(tmp_path):
    """include/lsg.h compiles as C99 with warnings as errors (the boundary has no C++ or torch
    types), and a C program links against the library's exported names."""
    import shutil
    import subprocess

    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    names = sorted(declared_functions())
    src = tmp_path / "use.c"
    body = "\n".join(f"    (void)&{n};" for n in names)
    src.write_text(f'#include "lsg.h"\nint main(void) {{\n{body}\n    return 0;\n}}\n')
    lib = Path(_lib.library()._name)
    cmd = [gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"), str(src), "-o",
           str(tmp_path / "use"), "-L", str(lib.parent), "-l:" + lib.name]
    done = subprocess.run(cmd, capture_output=True, text=True)
    assert done.returncode == 0, done.stderr


def _clifford_problem_walk(circuit, noise):
    """The Clifford check as a plain walk over the gates in order (the first problem found), by
    the oracle's own tables."""
    from oracle.clifford import clifford_problem

    return clifford_problem(circuit, noise)


def test_oracle_pauli_tables_and_branches_equal_the_engines():
    """The oracle's Clifford tables and Pauli branches (derived its own way) equal the host's for
    products of random Clifford gates on one to three qubits, refuse the same non-Clifford gates,
    and give the same branches and cumulative probabilities for Pauli channels."""
    from lucivant_sim_gb300.clifford import clifford_map, kind_of, pauli_noise
    from lucivant_sim_gb300.gates import GATES
    from lucivant_sim_gb300.noise import amplitude_damping, pauli_channel
    from oracle import clifford as oc

    rng = np.random.default_rng(5)
    names = [n for n in ("h", "s", "sdg", "x", "y", "z", "sx", "cx", "cz", "swap", "iswap", "ecr") if n in GATES]
    for trial in range(60):
        k = 1 + trial % 3
        u = np.eye(1 << k, dtype=np.complex128)
        for _ in range(5):
            name = names[int(rng.integers(len(names)))]
            spec = GATES[name]
            if spec.qubits > k:
                continue
            qs = [int(q) for q in rng.permutation(k)[: spec.qubits]]
            m = np.asarray(spec.build(), dtype=np.complex128)
            # embed on qubits qs (first qubit most significant) by permuting a kron with identity
            full = np.kron(m, np.eye(1 << (k - spec.qubits)))
            order = qs + [q for q in range(k) if q not in qs]
            t = full.reshape([2] * (2 * k))
            inv = np.argsort(order)
            t = t.transpose(list(inv) + [k + i for i in inv])
            u = t.reshape(1 << k, 1 << k) @ u
        mine, theirs = oc.conjugation_table(u), clifford_map(u)
        assert mine is not None and theirs is not None
        assert np.array_equal(mine.bits, theirs.bits) and np.array_equal(mine.sign, theirs.sign)
        assert oc.kind_of(mine) == kind_of(theirs)
    for name, params in (("t", ()), ("rx", (0.3,)), ("ccx", ()), ("u3", (0.1, 0.2, 0.3))):
        m = np.asarray(GATES[name].build(*params), dtype=np.complex128)
        assert oc.conjugation_table(m) is None and clifford_map(m) is None, name
    for ch in (depolarizing(1e-3), depolarizing(0.02, 2), pauli_channel({"X": 0.1, "Z": 0.05}),
               pauli_channel({"XY": 0.2, "ZI": 0.1})):
        a, b = oc.pauli_noise(ch), pauli_noise(ch)
        assert a is not None and b is not None
        assert a.branches == b.branches and np.array_equal(a.cumulative, b.cumulative)
    assert oc.pauli_noise(amplitude_damping(0.1)) is None and pauli_noise(amplitude_damping(0.1)) is None


def test_clifford_check_and_encoder_columns():
    """The columnar Clifford check reports the problem a walk over the gates finds first; the
    encoder's columns give every gate's qubits."""
    from lucivant_sim_gb300 import stabilizer as st
    from lucivant_sim_gb300.clifford import GateColumns, clifford_problem
    from lucivant_sim_gb300.noise import amplitude_damping, pauli_channel

    head = 'OPENQASM 3; include "stdgates.inc"; qubit[4] q; bit[4] c; '
    programs = [
        head + "h q[0]; cx q[0], q[1]; s q[2]; c = measure q;",
        head + "h q[0]; t q[1]; cx q[0], q[1]; rx(0.3) q[2];",
        head + "h q[0]; x q[3]; t q[1];",
        head + "x q[2]; ccx q[0], q[1], q[2]; h q[1];",
    ]
    models = [
        None,
        NoiseModel().add_gate_error(depolarizing(1e-3)),
        NoiseModel().add_gate_error(amplitude_damping(0.1), gates="x"),
        NoiseModel().add_gate_error(amplitude_damping(0.1), qubits=[1]).add_gate_error(pauli_channel({"Z": 0.1}), gates="h"),
        NoiseModel().add_gate_error(amplitude_damping(0.2), gates="h", qubits=[0]),
    ]
    for src in programs:
        c = ls.parse(src)
        for nm in models:
            assert clifford_problem(c, nm) == _clifford_problem_walk(c, nm), (src, nm)
    c = ls.parse(head + "h q[0]; cx q[3], q[1]; ccx q[0], q[1], q[2]; s q[2];")
    cols = GateColumns(st.all_gates(c.operations))
    assert cols.position(0).tolist() == [0, 3, 0, 2]
    assert cols.position(1).tolist() == [0, 1, 1, 0]
    assert cols.position(2).tolist() == [0, 0, 2, 0]
    assert cols.names == ["h", "cx", "ccx", "s"] and cols.arity.tolist() == [1, 2, 3, 1]


class _StandInRegister:
    """A register without a device: counts the bytes alive so a test can check a budget."""

    live = 0
    peak = 0
    lock = __import__("threading").Lock()

    def __init__(self, nbits: int, precision: int, batch: int = 1) -> None:
        from lucivant_sim_gb300 import serve

        self.nbits, self.precision, self.batch = nbits, precision, batch
        self.size = serve.register_bytes(nbits, precision, batch)
        with self.lock:
            type(self).live += self.size
            type(self).peak = max(type(self).peak, type(self).live)

    def free(self) -> None:
        with self.lock:
            type(self).live -= self.size
            self.size = 0


def _stand_in_server(monkeypatch, budget: int, run_s: float = 0.0, workers: int = 3):
    import time as _time

    from lucivant_sim_gb300 import serve

    _StandInRegister.live = _StandInRegister.peak = 0
    monkeypatch.setattr(_lib, "ensure_device", lambda *a, **k: None)
    monkeypatch.setattr(_lib, "mem_info", lambda: (1 << 40, 1 << 40))
    monkeypatch.setattr(_lib, "Register", _StandInRegister)
    seen: list[tuple[int, int]] = []

    def fake_execute(prep, precision, reg=None):
        seen.append((srv.used, _StandInRegister.live))
        _time.sleep(run_s)
        return {"values": np.zeros(prep["batch"])}

    monkeypatch.setattr(serve, "execute", fake_execute)
    srv = serve.Server(precision="c64", workers=workers, prep_workers=2, memory_bytes=budget)
    return srv, seen


def test_server_budget_covers_pooled_registers(monkeypatch):
    """Idle registers kept for reuse stay allocated: across jobs of many shapes, the bytes alive
    (running jobs' registers plus pooled ones) never exceed the server's budget, and the server's
    own count covers them."""
    from lucivant_sim_gb300 import serve

    budget = 192 << 20  # the 64 MiB program room per job lets about two jobs in at once
    srv, seen = _stand_in_server(monkeypatch, budget, run_s=0.01)
    jobs = []
    for i, (n, sweep) in enumerate([(14, 2), (15, 3), (16, 1), (14, 4), (17, 2), (15, 5), (16, 3), (18, 2)] * 2):
        names = [f"p{k}" for k in range(2 * n)]
        params = [dict(zip(names, np.random.default_rng(i + s).uniform(0, 6, 2 * n).tolist())) for s in range(sweep)]
        jobs.append(dict(kind="expect", arrival=0.0, qasm=wl.hea_template(n, 1), params=params,
                         observable={"Z" * n: 1.0}))  # fmt: skip
    try:
        out = serve.replay(jobs, srv, realtime=False)
        assert len(out["results"]) == len(jobs)
        assert _StandInRegister.peak <= budget
        for used, live in seen:
            assert used <= budget and live <= used
        assert srv.used == srv.pool.bytes == _StandInRegister.live
    finally:
        srv.close()
    assert _StandInRegister.live == 0 and srv.used == 0


def test_server_close_resolves_every_future(monkeypatch):
    """Closing the server with jobs still queued or in preparation resolves every future: run
    jobs with their result, the rest with RuntimeError('server closed')."""
    srv, _ = _stand_in_server(monkeypatch, 1 << 30, run_s=0.3, workers=1)
    futures = [srv.submit(dict(kind="expect", qasm=wl.hea_template(4, 1), observable={"ZZZZ": 1.0},
                               params=[{f"p{k}": 0.1 * k for k in range(8)}])) for _ in range(6)]  # fmt: skip
    import concurrent.futures as cf

    cf.wait(futures, timeout=120, return_when=cf.FIRST_COMPLETED)  # one job has run
    srv.close()
    for f in futures:
        assert f.done()
        exc = f.exception()
        assert exc is None or (isinstance(exc, RuntimeError) and "server closed" in str(exc))
    assert any(f.exception() is not None for f in futures)


def test_outcome_pair_space_deposits_like_orrery():
    """The device computes, per combination of reported pair bits, its probability (scatter of
    the marginal onto the pair bits, then each pair's readout flips); depositing that space onto
    classical bits gives the reference's branching result. Here the space is built on the host
    from the oracle's probabilities, for pairs that share a qubit and pairs that share a bit."""
    from lucivant_sim_gb300.circuit import final_measurements
    from lucivant_sim_gb300.noise import ReadoutError
    from lucivant_sim_gb300.simulator import deposit_pairs

    src = """OPENQASM 3.0; include "stdgates.inc"; qubit[4] q; bit[5] c;
    h q[0]; cx q[0], q[1]; ry(0.7) q[2]; cx q[2], q[3];
    c[0] = measure q[0]; c[1] = measure q[1]; c[2] = measure q[1]; c[2] = measure q[3]; c[4] = measure q[2];"""
    c = ls.parse(src)
    noise = NoiseModel().add_readout_error(ReadoutError(0.04, 0.09), qubits=[1]).add_readout_error(
        ReadoutError(0.2, 0.01), qubits=[3])
    pairs = final_measurements(c)
    measured = sorted({q for q, _ in pairs})
    pos = {q: i for i, q in enumerate(measured)}
    dist = dense.marginal(dense.probabilities_array(c, noise), c.num_qubits, measured)
    space = np.zeros(1 << len(pairs))
    for i, p in enumerate(dist):
        if p > 1e-12:
            space[sum(((i >> pos[q]) & 1) << j for j, (q, _) in enumerate(pairs))] = p
    for j, (q, _) in enumerate(pairs):
        err = noise.readout_error(q)
        if err is None:
            continue
        b = 1 << j
        for e in range(space.size):
            if not e & b:
                a0, a1 = space[e], space[e | b]
                space[e], space[e | b] = a0 * (1 - err.p01) + a1 * err.p10, a0 * err.p01 + a1 * (1 - err.p10)
    got = deposit_pairs(space, [cb for _, cb in pairs], c.num_clbits)
    want = dense.outcome_probabilities(c, noise)
    got = {ls.simulator.format_bits(c, k): v for k, v in got.items() if v > 1e-12}
    assert got.keys() == want.keys()
    assert all(abs(got[k] - v) < 1e-14 for k, v in want.items())


def _general_parse(src, params=None):
    """The general reader alone (token stream, every rule), for comparison with the fast path."""
    from lucivant_sim_gb300 import qasm

    r = qasm._Reader(src, params or {}, None)
    ops = r.program()
    s = r.scope
    extra = set(params or {}) - set(r.used)
    if extra:
        raise qasm.QasmError(f"the program has no input named {', '.join(sorted(extra))}")
    return qasm.Circuit(s.nq, s.nc, tuple(ops), tuple(s.qregs.values()), tuple(s.cregs.values()), dict(r.used))


def _same_circuit(a, b) -> None:
    assert (a.num_qubits, a.num_clbits, a.qregs, a.cregs) == (b.num_qubits, b.num_clbits, b.qregs, b.cregs)
    assert dict(getattr(a, "params", {}) or {}) == dict(getattr(b, "params", {}) or {})

    def same_ops(xs, ys) -> None:
        assert len(xs) == len(ys)
        for x, y in zip(xs, ys, strict=True):
            assert x.kind == y.kind
            if x.kind == "gate":
                assert (x.name, x.qubits, x.params) == (y.name, y.qubits, y.params)
                assert x.matrix.tobytes() == y.matrix.tobytes()
            elif x.kind == "if":
                assert x.condition == y.condition
                same_ops(x.then, y.then)
                same_ops(x.otherwise, y.otherwise)
            else:
                assert x == y

    same_ops(a.operations, b.operations)
    assert a.digest() == b.digest()


def test_plain_program_fast_path_reads_like_the_general_reader():
    """Plain programs (declarations, standard gates with number or input arguments on indexed
    qubits, measurements) are read without the token stream; the Circuit is the general reader's,
    operation for operation, and everything else still goes through the general reader."""
    from lucivant_sim_gb300 import qasm
    from lucivant_sim_gb300.gates import GATES

    rng = np.random.default_rng(8)
    programs = [(wl.brickwork(9, 7, seed=2), None), (wl.brickwork(5, 3, seed=4, measure=False), None),
                (wl.hea(6, 2, seed=3), None), (wl.clifford_layers(12, 3, seed=5), None)]  # fmt: skip
    names = {n: GATES[n].params for n in ("u3", "rx", "ry", "rz", "cx", "cz", "swap", "h", "sx", "U", "CX", "p", "rzz", "crx", "ccx")}
    for case in range(12):  # random plain programs: qreg/creg and qubit/bit spellings, inputs, measures
        n = int(rng.integers(3, 9))
        old = case % 2 == 0
        lines = ["OPENQASM 2.0;" if old else "OPENQASM 3.0;", 'include "qelib1.inc";' if old else 'include "stdgates.inc";']
        lines += [f"qreg q[{n}];", f"creg c[{n}];"] if old else [f"qubit[{n}] q;", f"bit[{n}] c;", "input float th;"]
        for _ in range(25):
            name = str(rng.choice(list(names)))
            k = GATES[name].qubits
            qs = ", ".join(f"q[{int(q)}]" for q in rng.permutation(n)[:k])
            args = [repr(float(v)) for v in rng.uniform(-4, 4, size=names[name])]
            if args and not old and rng.random() < 0.3:
                args[0] = "-th" if rng.random() < 0.5 else "th"
            lines.append(f"{name}({', '.join(args)}) {qs};" if args else f"{name} {qs};")
        lines.append(f"c[{int(rng.integers(n))}] = measure q[{int(rng.integers(n))}];" if case % 3 else "c = measure q;")
        programs.append(("\n".join(lines) + "\n", None if old else {"th": float(rng.uniform(-1, 1))}))
    programs.append((wl.hea_template(5, 2), {f"p{k}": 0.25 * k - 1 for k in range(20)}))
    for src, params in programs:
        assert qasm._fast_parse(src, params or {}) is not None, src[:200]
        _same_circuit(qasm.parse(src, params), _general_parse(src, params))
    # not plain: the general reader (same Circuit, by construction)
    for src in (wl.midcircuit(8, 1, seed=1), "OPENQASM 3; qubit[2] q; h q; // broadcast\n",
                "OPENQASM 3; qubit[2] q; rx(pi/2) q[0]; cx q[0], q[1];", "OPENQASM 3; qubit[3] q; inv @ s q[1];"):  # fmt: skip
        assert qasm._fast_parse(src, {}) is None
        _same_circuit(qasm.parse(src), _general_parse(src))
    # errors are the general reader's
    bad = ["OPENQASM 3; qubit[2] q; cx q[0];", "OPENQASM 3; qubit[2] q; cx q[0], q[0];", "OPENQASM 3; qubit[2] q; h q[2];",
           "OPENQASM 3; qubit[2] q; u3(1, 2) q[0];", "OPENQASM 3; qubit[2] q; foo q[0];",
           "OPENQASM 3; input float a; qubit[1] q; rx(a) q[0];", "OPENQASM 3; qubit[0] q;"]  # fmt: skip
    for src in bad:
        with pytest.raises(qasm.QasmError) as fast_err:
            qasm.parse(src)
        with pytest.raises(qasm.QasmError) as general_err:
            _general_parse(src)
        assert str(fast_err.value) == str(general_err.value)
    with pytest.raises(qasm.QasmError, match="no input named"):
        qasm.parse("OPENQASM 3; qubit[1] q; h q[0];", {"zz": 1.0})


def test_jobs_of_one_structure_combine_into_one_table():
    """Served jobs with the same operator structure (here brickwork circuits of one width and
    depth, other angles and seeds) get one structure key, and their combined table gives each
    member exactly its own job's operators: shared data once, differing data per member."""
    from lucivant_sim_gb300 import serve

    jobs = [dict(kind="sample", qasm=wl.brickwork(7, 5, seed=s), shots=100, seed=s) for s in (1, 2, 3)]
    jobs.append(dict(kind="sample", qasm=wl.brickwork(7, 6, seed=4), shots=100, seed=4))
    preps = [serve.prepare(j) for j in jobs]
    assert preps[0]["key"] == preps[1]["key"] == preps[2]["key"] != preps[3]["key"]
    table, flat = serve.combined_ops(preps[:3])
    pool = flat.view(np.complex128)
    shared = int((table["batch_stride"] == 0).sum())
    assert 0 < shared < len(table)  # cx (and any equal gates) once, the u3 of each job per member
    for b, prep in enumerate(preps[:3]):
        t0, f0 = prep["ops"]
        p0 = f0.view(np.complex128)
        starts = t0["data"]
        ends = np.append(starts[1:], p0.size)
        for i in range(len(t0)):
            size = ends[i] - starts[i]
            at = table[i]["data"] + b * table[i]["batch_stride"]
            assert np.array_equal(pool[at:at + size], p0[starts[i]:ends[i]])
            assert (t0[i]["kind"], t0[i]["nbits"], tuple(t0[i]["bits"])) == (table[i]["kind"], table[i]["nbits"], tuple(table[i]["bits"]))


def test_cgates_from_kinds_fills_and_refuses():
    """The library's gate-record filler for columnar circuits: per-kind fields, qubits of the
    used slots, zeros elsewhere; bad kinds, widths and qubits refused (host only)."""
    from lucivant_sim_gb300 import stabilizer as st

    lib = st._lib_stab()
    kind = np.array([1, 0, 1], dtype=np.int64)
    code = np.array([5, 7], dtype=np.int16)
    nq = np.array([1, 2], dtype=np.int16)
    noise = np.array([-1, 3], dtype=np.int16)
    q = np.array([[4, -1, -1], [2, 9, -1], [0, -1, -1]], dtype=np.int64)
    ar = np.array([1, 2, 1], dtype=np.int64)
    out = np.zeros(3, dtype=st.CGATE)
    assert lib.lsg_cgates_from_kinds(3, kind.ctypes.data, 2, code.ctypes.data, nq.ctypes.data, noise.ctypes.data,
                                     q.ctypes.data, ar.ctypes.data, out.ctypes.data) == 0  # fmt: skip
    assert out["code"].tolist() == [7, 5, 7] and out["nq"].tolist() == [2, 1, 2] and out["noise"].tolist() == [3, -1, 3]
    assert out["a"].tolist() == [4, 2, 0] and out["b"].tolist() == [0, 9, 0] and out["c"].tolist() == [0, 0, 0]
    for bad_kind, bad_ar, bad_q in ((2, 1, 4), (0, 4, 4), (0, 1, -3)):
        k2, a2, q2 = kind.copy(), ar.copy(), q.copy()
        k2[0], a2[0], q2[0, 0] = bad_kind, bad_ar, bad_q
        rc = lib.lsg_cgates_from_kinds(3, k2.ctypes.data, 2, code.ctypes.data, nq.ctypes.data, noise.ctypes.data,
                                       q2.ctypes.data, a2.ctypes.data, out.ctypes.data)  # fmt: skip
        assert rc == _lib.LSG_E_ARG


def test_run_takes_a_columnar_circuit_without_building_its_operations(monkeypatch):
    """ls.run recognises a columnar circuit as a circuit without asking for its operation objects
    (4.1 M of them at the 2048-qubit config), and the stabilizer choice reads its columns."""
    from lucivant_sim_gb300 import circuit as circ, simulator

    col = wl.clifford_layers_circuit(64, 5, seed=1)

    def refuse(self):
        raise AssertionError("operations built")

    monkeypatch.setattr(circ.ColumnarCircuit, "operations", property(refuse))
    assert simulator.to_circuit(col) is col
    assert simulator.choose_method(col, wl.stabilizer_noise(1e-3), "automatic") == "stabilizer"


def test_columnar_clifford_circuit_is_the_parsed_circuit():
    """The wide Clifford workload held as arrays is the circuit its OpenQASM text parses to
    (digest, operations, final measurements), and its gate columns give the stabilizer encoder
    and the Clifford check exactly what the parsed circuit's gate objects give."""
    from lucivant_sim_gb300 import stabilizer as st
    from lucivant_sim_gb300.clifford import clifford_problem, gates_and_columns

    for n, layers, seed in ((16, 3, 3), (65, 7, 2)):
        col = wl.clifford_layers_circuit(n, layers, seed=seed)
        ref = ls.parse(wl.clifford_layers(n, layers, seed=seed))
        assert col.digest() == ref.digest() and col.count_ops() == ref.count_ops()
        assert col.final_measurements() == ref.final_measurements() and not col.is_dynamic()
        g1, c1 = gates_and_columns(col)
        g2, c2 = gates_and_columns(ref)
        assert c1.names == c2.names and c1.qubits == c2.qubits and np.array_equal(c1.arity, c2.arity)
        for j in range(3):
            assert np.array_equal(c1.position(j), c2.position(j))
        for a, b in zip(c1.name_arity_groups, c2.name_arity_groups, strict=True):
            assert np.array_equal(a, b)
        # the same gates share a matrix (each gate's group named by the group's first gate)
        assert np.array_equal(c1.matrix_groups[0][c1.matrix_groups[1]], c2.matrix_groups[0][c2.matrix_groups[1]])
        for noise in (wl.stabilizer_noise(1e-2), None):
            assert clifford_problem(col, noise, g1, c1) == clifford_problem(ref, noise, g2, c2)
            assert st._has_gate_noise(g1, noise, c1) == st._has_gate_noise(g2, noise, c2)
            e1 = st.Encoder(noise).encode(g1, noise is not None, c1)
            e2 = st.Encoder(noise).encode(g2, noise is not None, c2)
            assert np.array_equal(e1, e2)
        assert [g.qubits for g in g1[:5]] == [g.qubits for g in g2[:5]] and len(g1) == len(g2)


def test_autotuner_cache_is_per_build_and_survives_a_choice_that_no_longer_plans(tmp_path, monkeypatch):
    """With a stand-in program (no device): the fastest candidate is kept in the file; an entry
    whose choice a later build refuses is searched again instead of failing the run; another
    build or device keys its choices apart."""
    from types import SimpleNamespace

    from lucivant_sim_gb300 import autotune

    monkeypatch.setenv("LSG_TUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "_identity", "build-a")
    monkeypatch.setattr(autotune, "_memory", {})
    reg = SimpleNamespace(nbits=24, precision=_lib.R64, batch=4)
    ops = SimpleNamespace(rows=[(0, 2, (0, 12), 0, 0), (2, 4, (0, 1, 12, 13), 16, 0)])

    class FakeProgram:
        refuse: set = set()

        def __init__(self, reg, ops, opts=None):
            key = None if opts is None else (opts.tile_bits, opts.ctas)
            if key in FakeProgram.refuse:
                raise ValueError("the plan does not fit")
            self.key, self.passes, self.specialized = key, 3, True

        def run_from_basis(self, reg, index, timed=False):
            # larger tiles and fewer CTAs are faster here
            return np.array([10.0 - self.key[0] * 0.5 + self.key[1] * 0.1])

        def free(self):
            pass

    monkeypatch.setattr(_lib, "Program", FakeProgram)
    prog, info = autotune.tuned_program(reg, ops)
    assert not info["cached"] and len(info["candidates"]) == 4
    best = prog.key
    cands = [(c.tile_bits, c.ctas) for c in autotune.candidates(24, _lib.R64)]
    assert best == (max(k for k, _ in cands), min(c for _, c in cands))
    key_a = autotune.shape_key(reg, ops)
    assert list(__import__("json").loads((tmp_path / "tune.json").read_text())) == [key_a]
    autotune._memory.clear()  # a later process finds it in the file
    prog, info = autotune.tuned_program(reg, ops)
    assert info["cached"] and prog.key == best
    autotune._memory.clear()
    FakeProgram.refuse = {best}  # a later build refuses the kept choice: searched again
    prog, info = autotune.tuned_program(reg, ops)
    assert not info["cached"] and prog.key != best and prog.key is not None
    monkeypatch.setattr(autotune, "_identity", "build-b")
    assert autotune.shape_key(reg, ops) != key_a
    assert not list(tmp_path.glob("*.tmp"))


def test_accelerator_methods_are_refused_as_orrery_refuses_them():
    """Orrery's opt-in accelerator methods: the method-choice checks come first (a noisy circuit
    gets the statevector misfit message), then the seed check, then the missing package's
    message; no device call is made on the way."""
    bell = 'OPENQASM 3; include "stdgates.inc"; qubit[2] q; bit[2] c; h q[0]; cx q[0], q[1]; c = measure q;'
    for method, extra, module in (("statevector_aer", "Qiskit Aer", "qiskit_aer"), ("stabilizer_stim", "Stim", "stim")):
        try:
            __import__(module)
        except ImportError:
            with pytest.raises(ls.SimulationError, match=f"this method needs {extra}: pip install lucivant-sim\\[accel\\]"):
                ls.run(bell, shots=10, seed=1, method=method)
        with pytest.raises(ValueError, match="seed must not be negative"):
            ls.run(bell, shots=10, seed=-1, method=method)
    with pytest.raises(ls.SimulationError, match="runs ideal circuits without mid-circuit measurement"):
        ls.run(bell, shots=10, seed=1, method="statevector_aer", noise=NoiseModel.uniform(single=0.01))
    with pytest.raises(ls.SimulationError, match="stabilizer_stim runs ideal circuits"):
        ls.run(bell, shots=10, seed=1, method="stabilizer_stim", noise=NoiseModel.uniform(single=0.01))
