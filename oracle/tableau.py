"""Oracle (test infrastructure): NumPy restatement of Orrery's stabilizer engine
(``src/lucivant_sim/stabilizer.py``). Not shipped; never called by the product.

Layout as in the reference (``stabilizer.py:193-208``): ``x[q, row]``, ``z[q, row]`` uint8 with
rows 0..n-1 destabilizers and n..2n-1 stabilizers, ``r[row]`` the sign bit.
"""

from __future__ import annotations

from typing import Any

import numpy as np
from numpy.typing import NDArray

from oracle.clifford import clifford_problem, kind_of, pauli_noise
from oracle.clifford import conjugation_table as clifford_map

U8 = NDArray[np.uint8]


class Tableau:
    def __init__(self, n: int) -> None:
        self.n = n
        self.x = np.zeros((n, 2 * n), dtype=np.uint8)
        self.z = np.zeros((n, 2 * n), dtype=np.uint8)
        self.r = np.zeros(2 * n, dtype=np.uint8)
        i = np.arange(n)
        self.x[i, i] = 1
        self.z[i, i + n] = 1

    def copy(self) -> Tableau:
        t = Tableau.__new__(Tableau)
        t.n, t.x, t.z, t.r = self.n, self.x.copy(), self.z.copy(), self.r.copy()
        return t

    def apply(self, cmap: Any, qubits: tuple[int, ...]) -> None:
        """Named fast rules (``stabilizer.py:224-254``) or the table (``:256-264``)."""
        kind = kind_of(cmap)
        x, z, r = self.x, self.z, self.r
        a = qubits[0]
        if kind is None:
            idx = np.zeros(2 * self.n, dtype=np.int64)
            for q in qubits:
                idx = (idx << 2) | (x[q].astype(np.int64) << 1) | z[q]
            new = cmap.bits[idx]
            r ^= cmap.sign[idx]
            for i, q in enumerate(qubits):
                x[q] = new[:, 2 * i]
                z[q] = new[:, 2 * i + 1]
        elif kind == "h":
            r ^= x[a] & z[a]
            x[a], z[a] = z[a].copy(), x[a].copy()
        elif kind == "s":
            r ^= x[a] & z[a]
            z[a] ^= x[a]
        elif kind == "sdg":
            r ^= x[a] & (z[a] ^ 1)
            z[a] ^= x[a]
        elif kind == "x":
            r ^= z[a]
        elif kind == "z":
            r ^= x[a]
        elif kind == "y":
            r ^= x[a] ^ z[a]
        elif kind == "cx":
            b = qubits[1]
            r ^= x[a] & z[b] & (x[b] ^ z[a] ^ 1)
            x[b] ^= x[a]
            z[a] ^= z[b]
        elif kind == "cz":
            b = qubits[1]
            r ^= x[a] & x[b] & (z[a] ^ z[b])
            z[a] ^= x[b]
            z[b] ^= x[a]

    def pauli(self, label: Any, qubits: tuple[int, ...]) -> None:
        for (px, pz), q in zip(label, qubits, strict=True):
            if px:
                self.r ^= self.z[q]
            if pz:
                self.r ^= self.x[q]

    def rowsum_into(self, targets: NDArray[np.int64], src: int) -> None:
        """Row[t] := Row[src]·Row[t] with the phase exponent summed mod 4 (``stabilizer.py:276-286``)."""
        if len(targets) == 0:
            return
        xs = self.x[:, src].astype(np.int8)[:, None]
        zs = self.z[:, src].astype(np.int8)[:, None]
        xt = self.x[:, targets].astype(np.int8)
        zt = self.z[:, targets].astype(np.int8)
        g = (xs & zs) * (zt - xt) + (xs & (1 - zs)) * (zt * (2 * xt - 1)) + ((1 - xs) & zs) * (xt * (1 - 2 * zt))
        tot = 2 * self.r[targets].astype(np.int64) + 2 * int(self.r[src]) + g.sum(axis=0, dtype=np.int64)
        self.r[targets] = (np.mod(tot, 4) == 2).astype(np.uint8)
        self.x[:, targets] ^= self.x[:, src][:, None]
        self.z[:, targets] ^= self.z[:, src][:, None]

    def deterministic(self, a: int) -> int:
        """``stabilizer.py:288-301``."""
        n = self.n
        sx = np.zeros(n, dtype=np.int8)
        sz = np.zeros(n, dtype=np.int8)
        sr = 0
        for i in np.flatnonzero(self.x[a, :n]):
            row = int(i) + n
            xs, zs = self.x[:, row].astype(np.int8), self.z[:, row].astype(np.int8)
            g = (xs & zs) * (sz - sx) + (xs & (1 - zs)) * (sz * (2 * sx - 1)) + ((1 - xs) & zs) * (sx * (1 - 2 * sz))
            sr = 1 if (2 * sr + 2 * int(self.r[row]) + int(g.sum())) % 4 == 2 else 0
            sx ^= xs
            sz ^= zs
        return sr

    def measure(self, a: int, rng: Any = None, forced: int | None = None) -> int:
        """``stabilizer.py:303-327``: first stabilizer with x[a] = 1 is the pivot."""
        n = self.n
        cand = np.flatnonzero(self.x[a, n:])
        if len(cand) == 0:
            return self.deterministic(a)
        p = int(cand[0]) + n
        others = np.flatnonzero(self.x[a])
        self.rowsum_into(others[others != p], p)
        self.x[:, p - n] = self.x[:, p]
        self.z[:, p - n] = self.z[:, p]
        self.r[p - n] = self.r[p]
        self.x[:, p] = 0
        self.z[:, p] = 0
        self.z[a, p] = 1
        out = forced if forced is not None else int(rng.integers(2))
        self.r[p] = out
        return out

    def reset(self, a: int, rng: Any) -> None:
        if self.measure(a, rng):
            self.pauli([(1, 0)], (a,))

    def support(self, qubits: list[int]) -> tuple[U8, U8]:
        """(x0, basis) by packed GF(2) elimination (``stabilizer.py:333-365``)."""
        n = self.n
        sx = pack_rows(self.x[:, n:].T)
        sz = pack_rows(self.z[:, n:].T)
        sr = self.r[n:].copy()
        pivots: list[int] = []
        used = np.zeros(n, dtype=bool)
        for q in range(n):
            w, bit = q // 64, np.uint64(1) << np.uint64(q % 64)
            has = (sx[:, w] & bit) != 0
            cand = np.flatnonzero(has & ~used)
            if len(cand) == 0:
                continue
            p = int(cand[0])
            used[p] = True
            pivots.append(p)
            tg = np.flatnonzero(has)
            tg = tg[tg != p]
            if len(tg):
                rowsum_packed(sx, sz, sr, tg, p)
        x_full = solve_z(sz[~used], sr[~used], n)
        idx = np.asarray(qubits, dtype=np.int64)
        x0 = x_full[idx]
        vec = unpack_rows(sx[pivots], n)[:, idx] if pivots else np.zeros((0, len(idx)), dtype=np.uint8)
        if len(idx) == n and np.array_equal(idx, np.arange(n)):
            return x0, vec
        return x0, row_basis(vec)


def pack_rows(bits: U8) -> NDArray[np.uint64]:
    packed = np.packbits(np.ascontiguousarray(bits, dtype=np.uint8), axis=1, bitorder="little")
    pad = (-packed.shape[1]) % 8
    if pad:
        packed = np.pad(packed, ((0, 0), (0, pad)))
    return np.ascontiguousarray(packed).view(np.uint64)


def unpack_rows(words: NDArray[np.uint64], n: int) -> U8:
    return np.unpackbits(np.ascontiguousarray(words).view(np.uint8), axis=1, bitorder="little")[:, :n]


def rowsum_packed(sx: Any, sz: Any, sr: Any, targets: Any, p: int) -> None:
    """Packed rowsum with popcount phase masks (``stabilizer.py:381-395``)."""
    x1, z1 = sx[p], sz[p]
    x2, z2 = sx[targets], sz[targets]
    plus = (x1 & z1 & ~x2 & z2) | (x1 & ~z1 & x2 & z2) | (~x1 & z1 & x2 & ~z2)
    minus = (x1 & z1 & x2 & ~z2) | (x1 & ~z1 & ~x2 & z2) | (~x1 & z1 & x2 & z2)
    g = np.bitwise_count(plus).sum(axis=1, dtype=np.int64) - np.bitwise_count(minus).sum(axis=1, dtype=np.int64)
    tot = 2 * sr[targets].astype(np.int64) + 2 * int(sr[p]) + g
    sr[targets] = (np.mod(tot, 4) == 2).astype(np.uint8)
    sx[targets] ^= x1
    sz[targets] ^= z1


def solve_z(rows: Any, rhs: Any, n: int) -> U8:
    """One solution of rows·x = rhs, free variables 0 (``stabilizer.py:398-422``)."""
    m = rows.copy()
    b = rhs.astype(np.uint8).copy()
    x = np.zeros(n, dtype=np.uint8)
    piv: list[tuple[int, int]] = []
    used = np.zeros(len(m), dtype=bool)
    for q in range(n):
        w, bit = q // 64, np.uint64(1) << np.uint64(q % 64)
        has = (m[:, w] & bit) != 0
        cand = np.flatnonzero(has & ~used)
        if len(cand) == 0:
            continue
        p = int(cand[0])
        used[p] = True
        piv.append((q, p))
        o = np.flatnonzero(has)
        o = o[o != p]
        m[o] ^= m[p]
        b[o] ^= b[p]
    for q, p in piv:
        x[q] = b[p]
    return x


def row_basis(rows: U8) -> U8:
    """``stabilizer.py:425-440``."""
    m = rows.copy()
    basis = []
    for col in range(m.shape[1]):
        pv = np.flatnonzero(m[:, col])
        if len(pv) == 0:
            continue
        row = m[int(pv[0])].copy()
        basis.append(row)
        m[m[:, col].astype(bool)] ^= row
        if len(basis) == m.shape[1]:
            break
    return np.array(basis, dtype=np.uint8).reshape(len(basis), rows.shape[1])


def _gates(ops: Any) -> list[Any]:
    out: list[Any] = []
    for op in ops:
        if op.kind == "gate":
            out.append(op)
        elif op.kind == "if":
            out += _gates(op.then) + _gates(op.otherwise)
    return out


def _noisy(circuit: Any, noise: Any) -> bool:
    return noise is not None and any(noise.gate_error(g.name, g.qubits) is not None for g in _gates(circuit.operations))


def run_counts(circuit: Any, shots: int, noise: Any, rng: np.random.Generator) -> dict[int, int]:
    """Dispatch as ``stabilizer.py:495-511``."""
    problem = clifford_problem(circuit, noise)
    if problem:
        raise RuntimeError(problem)
    if shots == 0 or circuit.num_clbits == 0:
        return {}
    if circuit.is_dynamic():
        return per_shot(circuit, shots, noise, rng)
    if _noisy(circuit, noise):
        return frames(circuit, shots, noise, rng)
    return sampled(circuit, shots, noise, rng)


def reference_tableau(circuit: Any) -> Tableau:
    t = Tableau(circuit.num_qubits)
    for op in circuit.operations:
        if op.kind == "gate":
            t.apply(clifford_map(op.matrix), op.qubits)
    return t


def frame_gate(fx: U8, fz: U8, cmap: Any, qubits: tuple[int, ...]) -> None:
    """``stabilizer.py:566-594``."""
    kind = kind_of(cmap)
    a = qubits[0]
    if kind in ("x", "y", "z", "id"):
        return
    if kind == "h":
        fx[a], fz[a] = fz[a].copy(), fx[a].copy()
    elif kind in ("s", "sdg"):
        fz[a] ^= fx[a]
    elif kind == "cx":
        b = qubits[1]
        fx[b] ^= fx[a]
        fz[a] ^= fz[b]
    elif kind == "cz":
        b = qubits[1]
        fz[a] ^= fx[b]
        fz[b] ^= fx[a]
    else:
        idx = np.zeros(fx.shape[1], dtype=np.int64)
        for q in qubits:
            idx = (idx << 2) | (fx[q].astype(np.int64) << 1) | fz[q]
        new = cmap.bits[idx]
        for i, q in enumerate(qubits):
            fx[q] = new[:, 2 * i]
            fz[q] = new[:, 2 * i + 1]


def frames(circuit: Any, shots: int, noise: Any, rng: np.random.Generator) -> dict[int, int]:
    """Pauli frames over all shots (``stabilizer.py:514-563``)."""
    n = circuit.num_qubits
    ref = reference_tableau(circuit)
    pairs = circuit.final_measurements()
    if not pairs:
        return {}
    measured = sorted({q for q, _ in pairs})
    x0, _ = ref.support(measured)
    fx = np.zeros((n, shots), dtype=np.uint8)
    fz = rng.integers(0, 2, size=(n, shots), dtype=np.uint8)
    for op in circuit.operations:
        if op.kind != "gate":
            continue
        frame_gate(fx, fz, clifford_map(op.matrix), op.qubits)
        ch = noise.gate_error(op.name, op.qubits) if noise else None
        if ch is None:
            continue
        br = pauli_noise(ch)
        picks = np.minimum(np.searchsorted(br.cumulative, rng.random(shots), side="right"), len(br.branches) - 1)
        for b, label in enumerate(br.branches):
            if not any(px or pz for px, pz in label):
                continue
            mask = picks == b
            if not mask.any():
                continue
            for (px, pz), q in zip(label, op.qubits, strict=True):
                if px:
                    fx[q, mask] ^= 1
                if pz:
                    fz[q, mask] ^= 1
    pos = {q: i for i, q in enumerate(measured)}
    bits = np.stack([fx[q] ^ x0[pos[q]] for q in measured], axis=1)
    return count(circuit, pairs, pos, bits, noise, rng, shots)


def _pack(bits: U8, words: int) -> NDArray[np.uint64]:
    out = np.zeros(words, dtype=np.uint64)
    for i in np.flatnonzero(bits):
        out[i // 64] |= np.uint64(1) << np.uint64(i % 64)
    return out


def sampled(circuit: Any, shots: int, noise: Any, rng: np.random.Generator) -> dict[int, int]:
    """Ideal static: x0 plus random combinations of the basis (``stabilizer.py:597-619``)."""
    t = reference_tableau(circuit)
    pairs = circuit.final_measurements()
    if not pairs:
        return {}
    measured = sorted({q for q, _ in pairs})
    pos = {q: i for i, q in enumerate(measured)}
    x0, basis = t.support(measured)
    m = len(measured)
    words = (m + 63) // 64
    outs = np.repeat(_pack(x0, words)[None, :], shots, axis=0)
    if len(basis):
        coef = rng.integers(0, 2, size=(shots, len(basis)), dtype=np.uint8).astype(bool)
        packed = np.stack([_pack(row, words) for row in basis])
        for i in range(len(basis)):
            outs[coef[:, i]] ^= packed[i]
    bits = np.unpackbits(outs.view(np.uint8), axis=1, bitorder="little")[:, :m]
    return count(circuit, pairs, pos, bits, noise, rng, shots)


def count(circuit: Any, pairs: Any, pos: Any, bits: U8, noise: Any, rng: Any, shots: int) -> dict[int, int]:
    """Readout flips per pair, then counts (``stabilizer.py:622-643``)."""
    cl = np.zeros((shots, circuit.num_clbits), dtype=np.uint8)
    for q, c in pairs:
        val = bits[:, pos[q]]
        err = noise.readout_error(q) if noise else None
        if err is not None and (err.p01 or err.p10):
            val = val ^ (rng.random(shots) < np.where(val == 1, err.p10, err.p01)).astype(np.uint8)
        cl[:, c] = val
    packed = np.packbits(cl, axis=1, bitorder="little")
    rows, cnt = np.unique(packed, axis=0, return_counts=True)
    return {int.from_bytes(row.tobytes(), "little"): int(k) for row, k in zip(rows, cnt, strict=True)}


def per_shot(circuit: Any, shots: int, noise: Any, rng: np.random.Generator) -> dict[int, int]:
    """One tableau per shot after the shared noiseless prefix (``stabilizer.py:653-694``)."""
    ops = circuit.operations
    prefix = Tableau(circuit.num_qubits)
    start = 0
    for op in ops:
        if op.kind == "gate" and (noise is None or noise.gate_error(op.name, op.qubits) is None):
            prefix.apply(clifford_map(op.matrix), op.qubits)
            start += 1
        elif op.kind in ("barrier", "gphase"):
            start += 1
        else:
            break
    rest = ops[start:]
    tally: dict[int, int] = {}
    for _ in range(shots):
        st = prefix.copy()
        cl = [0] * circuit.num_clbits
        _run_ops(st, rest, cl, noise, rng)
        key = sum(b << i for i, b in enumerate(cl))
        tally[key] = tally.get(key, 0) + 1
    return tally


def _run_ops(st: Tableau, ops: Any, cl: list[int], noise: Any, rng: Any) -> None:
    for op in ops:
        k = op.kind
        if k == "gate":
            st.apply(clifford_map(op.matrix), op.qubits)
            ch = noise.gate_error(op.name, op.qubits) if noise else None
            if ch is not None:
                br = pauli_noise(ch)
                pick = int(np.searchsorted(br.cumulative, rng.random(), side="right"))
                st.pauli(br.branches[min(pick, len(br.branches) - 1)], op.qubits)
        elif k == "measure":
            out = st.measure(op.qubit, rng)
            err = noise.readout_error(op.qubit) if noise else None
            if err is not None and rng.random() < (err.p10 if out else err.p01):
                out ^= 1
            if op.clbit is not None:
                cl[op.clbit] = out
        elif k == "reset":
            st.reset(op.qubit, rng)
        elif k == "if":
            _run_ops(st, op.then if op.condition.holds(cl) else op.otherwise, cl, noise, rng)
