"""The stabilizer method on the device: run_counts with Orrery's dispatch
(``src/lucivant_sim/stabilizer.py:495-511``) — ideal static circuits sampled from the support,
noisy static circuits by Pauli frames, dynamic circuits one tableau per shot.

The draws come from the run's PCG64 stream: the device regenerates it bit for bit from the
generator's state, in Orrery's order, and the host generator is advanced past them afterwards,
so counts are identical to Orrery's for the same seed.
"""

from __future__ import annotations

import ctypes as C
from typing import Any

import numpy as np

from lucivant_sim_gb300 import _lib
from lucivant_sim_gb300._lib import SimulationError, check, library
from lucivant_sim_gb300.clifford import (
    GateColumns,
    all_gates,
    clifford_map,
    clifford_problem,
    first_index,
    gates_and_columns,
    kind_of,
    pauli_noise,
)

CODES = {"id": 0, "h": 1, "s": 2, "sdg": 3, "x": 4, "y": 5, "z": 6, "cx": 7, "cz": 8}

CGATE = np.dtype(
    [("code", "<i2"), ("noise", "<i2"), ("a", "<i2"), ("b", "<i2"), ("c", "<i2"), ("nq", "<i2"), ("pad", "<i4")]
)
NOISE = np.dtype([("k", "<i4"), ("nbranch", "<i4"), ("cumulative", "<f8", (16,)), ("label", "u1", (16,))])
assert CGATE.itemsize == 16 and NOISE.itemsize == 152

_SIGS = {
    "lsg_tab_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "lsg_tab_free": (C.c_int, [C.c_void_p]),
    "lsg_tab_apply": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int32]),
    "lsg_tab_download": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "lsg_tab_support": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.POINTER(C.c_int32)]),
    "lsg_frames_run": (C.c_int, [C.c_int, C.c_void_p, C.c_int64, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                 C.c_int64, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.POINTER(C.c_int64)]),
    "lsg_stab_sample": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_int32, C.c_int64, C.c_void_p, C.c_int32,
                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p,
                                  C.POINTER(C.c_int64)]),
    "lsg_pcg_raw": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]),
    "lsg_cgates_from_kinds": (C.c_int, [C.c_int64, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p]),
}  # fmt: skip


def _lib_stab() -> C.CDLL:
    lib = library()
    if not getattr(lib, "_stab_sigs", False):
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype, fn.argtypes = res, args
        lib._stab_sigs = True
    return lib


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


class Encoder:
    """Gate codes, conjugation tables and noise tables for the device (cached per matrix and per
    channel: circuits repeat their gates)."""

    def __init__(self, noise: Any) -> None:
        self.noise = noise
        self.tables: list[bytes] = []
        self.table_of: dict[bytes, int] = {}
        self.noise_rows: list[np.void] = []
        self.noise_of: dict[int, tuple[Any, int]] = {}
        self.code_by_id: dict[int, tuple[Any, int, int]] = {}
        # noise lookups depend on (name, qubits); without qubit-specific rules only on (name, arity)
        self.by_arity = noise is not None and all(r.qubits is None for r in getattr(noise, "rules", []))
        self.rule_cache: dict[tuple, Any] = {}

    def gate_code(self, g: Any) -> tuple[int, int]:
        hit = self.code_by_id.get(id(g.matrix))
        if hit is not None and hit[0] is g.matrix:
            return hit[1], hit[2]
        cmap = clifford_map(g.matrix)
        if cmap is None:  # pragma: no cover - clifford_problem refuses first
            raise SimulationError(f"{g.name} isn't a Clifford gate")
        kind = kind_of(cmap)
        if kind is not None:
            code, k = CODES[kind], cmap.k
        else:
            rec = bytearray(65)
            rec[0] = cmap.k
            for i in range(len(cmap.bits)):
                v = 0
                for bit in cmap.bits[i]:
                    v = (v << 1) | int(bit)
                rec[1 + i] = (int(cmap.sign[i]) << 7) | v
            key = bytes(rec)
            if key not in self.table_of:
                self.table_of[key] = len(self.tables)
                self.tables.append(key)
            code, k = 16 + self.table_of[key], cmap.k
        self.code_by_id[id(g.matrix)] = (g.matrix, code, k)
        return code, k

    def noise_code(self, g: Any) -> int:
        if self.noise is None:
            return -1
        key = (g.name, len(g.qubits)) if self.by_arity else (g.name, tuple(g.qubits))
        if key in self.rule_cache:
            ch = self.rule_cache[key]
        else:
            ch = self.rule_cache[key] = self.noise.gate_error(g.name, tuple(g.qubits))
        if ch is None:
            return -1
        hit = self.noise_of.get(id(ch))
        if hit is not None and hit[0] is ch:
            return hit[1]
        br = pauli_noise(ch)
        if br is None:  # pragma: no cover - refused earlier
            raise SimulationError(f"the {ch.name} noise isn't a Pauli channel")
        if len(br.branches) > 16 or ch.num_qubits > 2:
            raise SimulationError("Pauli noise with more than 16 branches or 2 qubits is not supported on the device")
        row = np.zeros((), dtype=NOISE)
        row["k"] = ch.num_qubits
        row["nbranch"] = len(br.branches)
        row["cumulative"][: len(br.cumulative)] = br.cumulative
        for i, label in enumerate(br.branches):
            v = 0
            for px, pz in label:
                v = (v << 2) | (px << 1) | pz
            row["label"][i] = v
        idx = len(self.noise_rows)
        self.noise_rows.append(row)
        self.noise_of[id(ch)] = (ch, idx)
        return idx

    def encode(self, gates: list[Any], with_noise: bool, cols: GateColumns | None = None) -> np.ndarray:
        n = len(gates)
        out = np.zeros(n, dtype=CGATE)
        if n == 0:
            return out
        # each distinct matrix and noise key once; per gate only C-level attribute reads
        # (map / attrgetter) into NumPy arrays
        cols = GateColumns(gates) if cols is None else cols
        first, inv = cols.matrix_groups
        codes = np.array([self.gate_code(gates[int(f)]) for f in first], dtype=np.int32).reshape(-1, 2)
        qmat = getattr(cols, "_qmat", None)
        if qmat is not None and (not with_noise or self.by_arity):
            # a columnar circuit: per kind (its distinct gates) the code, width and noise code, the
            # records filled by the library (same lookups in the same order as below)
            kind = np.ascontiguousarray(cols.matrix_ids, dtype=np.int64)
            nkinds = int(kind.max()) + 1
            group_kind = kind[first]
            kcode = np.zeros(nkinds, dtype=np.int16)
            knq = np.zeros(nkinds, dtype=np.int16)
            knoise = np.full(nkinds, -1, dtype=np.int16)
            kcode[group_kind], knq[group_kind] = codes[:, 0], codes[:, 1]
            if with_noise:
                kfirst, kinv = cols.name_arity_groups
                idx = np.array([self.noise_code(gates[int(f)]) for f in kfirst], dtype=np.int16)
                knoise[group_kind] = idx[kinv[first]]
            q = np.ascontiguousarray(qmat, dtype=np.int64)
            if q.ndim != 2 or q.shape[1] < 3:
                q = np.ascontiguousarray(np.pad(q.reshape(n, -1), ((0, 0), (0, 3 - q.reshape(n, -1).shape[1]))))
            arity = np.ascontiguousarray(cols.arity, dtype=np.int64)
            check(_lib_stab().lsg_cgates_from_kinds(n, _p(kind), nkinds, _p(kcode), _p(knq), _p(knoise), _p(q),
                                                    _p(arity), _p(out)))  # fmt: skip
            return out
        out["code"], out["nq"] = codes[inv, 0], codes[inv, 1]
        out["a"], out["b"], out["c"] = cols.position(0), cols.position(1), cols.position(2)
        if not with_noise:
            out["noise"] = -1
        elif self.by_arity:  # rules by gate name only: key (name, arity)
            kfirst, kinv = cols.name_arity_groups
            idx = np.array([self.noise_code(gates[int(f)]) for f in kfirst], dtype=np.int16)
            out["noise"] = idx[kinv]
        else:  # (name, qubits) keys: each distinct one looked up once
            keys = list(zip(cols.names, cols.qubits))
            code_of = {k: self.noise_code(gates[i]) for k, i in first_index(keys).items()}
            out["noise"] = np.fromiter(map(code_of.__getitem__, keys), dtype=np.int16, count=n)
        return out

    def table_bytes(self) -> np.ndarray:
        return np.frombuffer(b"".join(self.tables) or b"\0" * 65, dtype=np.uint8).copy()

    def noise_array(self) -> np.ndarray:
        return np.array(self.noise_rows, dtype=NOISE) if self.noise_rows else np.zeros(1, dtype=NOISE)


class Tableau:
    """A device tableau (Orrery's ``Tableau``)."""

    def __init__(self, n: int) -> None:
        _lib.ensure_device()
        self.lib = _lib_stab()
        self.n = n
        h = C.c_void_p()
        check(self.lib.lsg_tab_create(n, C.byref(h)))
        self.handle = h

    def apply(self, cg: np.ndarray, enc: Encoder) -> None:
        if len(cg):
            tables = enc.table_bytes()
            check(self.lib.lsg_tab_apply(self.handle, _p(cg), len(cg), _p(tables), len(enc.tables)))

    def arrays(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        n = self.n
        x = np.zeros((n, 2 * n), dtype=np.uint8)
        z = np.zeros((n, 2 * n), dtype=np.uint8)
        r = np.zeros(2 * n, dtype=np.uint8)
        check(self.lib.lsg_tab_download(self.handle, _p(x), _p(z), _p(r)))
        return x, z, r

    def support(self, qubits: list[int], want_basis: bool = True) -> tuple[np.ndarray, np.ndarray]:
        """(x0, basis) of the outcomes on ``qubits`` (``Tableau.support``)."""
        q = np.asarray(qubits, dtype=np.int32)
        m = len(q)
        x0 = np.zeros(m, dtype=np.uint8)
        rank = C.c_int32(0)
        basis = np.zeros((self.n, m), dtype=np.uint8) if want_basis else None  # rank <= n
        check(self.lib.lsg_tab_support(self.handle, _p(q), m, _p(x0), _p(basis) if basis is not None else None,
                                       C.byref(rank)))  # fmt: skip
        return x0, basis[: rank.value] if basis is not None else np.zeros((0, m), dtype=np.uint8)

    def free(self) -> None:
        if getattr(self, "handle", None):
            self.lib.lsg_tab_free(self.handle)
            self.handle = None

    def __del__(self) -> None:
        try:
            self.free()
        except Exception:
            pass


def rng_words(rng: np.random.Generator) -> np.ndarray:
    st = rng.bit_generator.state
    if st["bit_generator"] != "PCG64":
        raise ValueError("the stabilizer method needs numpy's PCG64 generator")
    if st["has_uint32"]:
        raise ValueError("the generator holds a buffered 32-bit value; start from a fresh generator")
    s, inc = st["state"]["state"], st["state"]["inc"]
    m = (1 << 64) - 1
    return np.array([s >> 64, s & m, inc >> 64, inc & m], dtype=np.uint64)


def advance_rng(rng: np.random.Generator, raw: int, n32_before: int) -> None:
    """Leave ``rng`` where NumPy leaves it after the same draws: ``raw`` 64-bit draws, of which
    the first uint32s (``n32_before`` of them, from uint8 integers) may leave a half buffered."""
    start = rng.bit_generator.state
    rng.bit_generator.advance(raw)
    if n32_before % 2:
        # the last integer draw split a 64-bit value: its high half stays buffered
        probe = np.random.PCG64()
        probe.state = start
        probe.advance(n32_before // 2)
        value = int(probe.random_raw(1)[0])
        st = rng.bit_generator.state
        st["has_uint32"] = 1
        st["uinteger"] = value >> 32
        rng.bit_generator.state = st


def _pairs(circuit: Any, noise: Any, measured: list[int]):
    pairs = circuit.final_measurements()
    pos = {q: i for i, q in enumerate(measured)}
    pq = np.array([q for q, _ in pairs], dtype=np.int32)
    pc = np.array([c for _, c in pairs], dtype=np.int32)
    ppos = np.array([pos[q] for q, _ in pairs], dtype=np.int32)
    perr = np.full(len(pairs), -1, dtype=np.int32)
    p01 = np.zeros(len(pairs))
    p10 = np.zeros(len(pairs))
    e = 0
    for j, (q, _c) in enumerate(pairs):
        err = noise.readout_error(q) if noise else None
        if err is not None and (err.p01 or err.p10):
            perr[j] = e
            p01[j], p10[j] = err.p01, err.p10
            e += 1
    return pairs, pq, pc, ppos, perr, p01, p10, e


def _count(bits: np.ndarray) -> dict[int, int]:
    """Counts of classical-bit rows (``stabilizer.py:641-643``)."""
    packed = np.packbits(bits, axis=1, bitorder="little")
    rows, cnt = np.unique(packed, axis=0, return_counts=True)
    return {int.from_bytes(row.tobytes(), "little"): int(k) for row, k in zip(rows, cnt, strict=True)}


def _has_gate_noise(gates: list[Any], noise: Any, cols: GateColumns | None = None) -> bool:
    """Whether any gate draws a noise channel. With rules by gate name only, each distinct (name,
    arity) is asked once, at its first gate."""
    if noise is None:
        return False
    if cols is not None and all(r.qubits is None for r in getattr(noise, "rules", [])):
        first = cols.name_arity_groups[0]
        return any(noise.gate_error(gates[int(i)].name, gates[int(i)].qubits) is not None for i in first)
    return any(noise.gate_error(g.name, g.qubits) is not None for g in gates)


def run_counts(circuit: Any, shots: int, noise: Any, rng: np.random.Generator) -> dict[int, int]:
    """Counts keyed by the classical bits as an integer (bit c = classical bit c)."""
    gates, cols = gates_and_columns(circuit)  # read once, shared by the Clifford check and the encoder
    problem = clifford_problem(circuit, noise, gates, cols)
    if problem:
        raise SimulationError(f"the stabilizer method runs Clifford circuits only: {problem}")
    n = circuit.num_qubits
    if shots == 0 or circuit.num_clbits == 0:
        if n > 0 and not circuit.is_dynamic() and not _has_gate_noise(gates, noise, cols):
            enc = Encoder(None)
            t = Tableau(n)
            t.apply(enc.encode(gates, False, cols), enc)
            t.free()
        return {}
    if circuit.is_dynamic():
        from lucivant_sim_gb300 import stabilizer_shots

        return stabilizer_shots.per_shot(circuit, shots, noise, rng)
    if _has_gate_noise(gates, noise, cols):
        return frames(circuit, shots, noise, rng, gates, cols)
    return sampled(circuit, shots, noise, rng, gates, cols)


def frames(circuit: Any, shots: int, noise: Any, rng: np.random.Generator, gates: list[Any] | None = None,
           cols: GateColumns | None = None) -> dict[int, int]:
    """Pauli frames for a static circuit with Pauli gate noise (``stabilizer.py:514-563``)."""
    lib = _lib_stab()
    n = circuit.num_qubits
    gates = all_gates(circuit.operations) if gates is None else gates
    pairs = circuit.final_measurements()
    if not pairs:
        return {}
    measured = sorted({q for q, _ in pairs})
    enc = Encoder(noise)
    cg = enc.encode(gates, True, cols)
    tables = enc.table_bytes()
    tab = Tableau(n)
    try:
        tab.apply(cg, enc)
        x0, _ = tab.support(measured, want_basis=False)
    finally:
        tab.free()
    _, pq, pc, ppos, perr, p01, p10, _nerr = _pairs(circuit, noise, measured)
    px0 = x0[ppos].astype(np.uint8)
    state = rng_words(rng)
    nt = enc.noise_array()
    bits = np.zeros((shots, circuit.num_clbits), dtype=np.uint8)
    raw = C.c_int64(0)
    check(lib.lsg_frames_run(n, _p(cg), len(cg), _p(tables), len(enc.tables), _p(nt), len(enc.noise_rows), shots,
                             _p(state), len(pq), _p(pq), _p(pc), _p(px0), _p(perr), _p(p01), _p(p10),
                             circuit.num_clbits, _p(bits), C.byref(raw)))  # fmt: skip
    advance_rng(rng, int(raw.value), -(-(n * shots) // 4))
    return _count(bits)


def sampled(circuit: Any, shots: int, noise: Any, rng: np.random.Generator, gates: list[Any] | None = None,
            cols: GateColumns | None = None) -> dict[int, int]:
    """Ideal static circuit: x0 plus random basis combinations (``stabilizer.py:597-619``)."""
    lib = _lib_stab()
    n = circuit.num_qubits
    gates = all_gates(circuit.operations) if gates is None else gates
    pairs = circuit.final_measurements()
    if not pairs:
        return {}
    measured = sorted({q for q, _ in pairs})
    enc = Encoder(None)
    cg = enc.encode(gates, False, cols)
    tab = Tableau(n)
    try:
        tab.apply(cg, enc)
        x0, basis = tab.support(measured, want_basis=True)
    finally:
        tab.free()
    _, _pq, pc, ppos, perr, p01, p10, _nerr = _pairs(circuit, noise, measured)
    nb = len(basis)
    basis_c = np.ascontiguousarray(basis if nb else np.zeros((1, len(measured)), dtype=np.uint8))
    state = rng_words(rng)
    bits = np.zeros((shots, circuit.num_clbits), dtype=np.uint8)
    raw = C.c_int64(0)
    check(lib.lsg_stab_sample(len(measured), _p(x0), _p(basis_c), nb, shots, _p(state), len(pc), _p(ppos), _p(pc),
                              _p(perr), _p(p01), _p(p10), circuit.num_clbits, _p(bits), C.byref(raw)))  # fmt: skip
    advance_rng(rng, int(raw.value), -(-(shots * nb) // 4) if nb else 0)
    return _count(bits)


def pcg_raw(rng: np.random.Generator, index: int) -> int:
    """The library's own PCG64: raw draw number ``index`` of ``rng`` (host code, no device)."""
    out = C.c_uint64(0)
    check(_lib_stab().lsg_pcg_raw(_p(rng_words(rng)), index, C.byref(out)))
    return int(out.value)
