"""ctypes binding of the engine library (``liblsg.so``, declared in ``include/lsg.h``).

Status codes map back to the exception types Orrery raises: bad arguments to ``ValueError``,
capacity misfits to :class:`SimulationError`, device allocation failures to ``MemoryError``.
The library must be built (``python -m lucivant_sim_gb300.build``); there is no CPU fallback, so a
missing library or GPU is an error, not a slower path.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path
from typing import Any

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "liblsg.so"

LSG_OK, LSG_E_ARG, LSG_E_CAPACITY, LSG_E_MEMORY, LSG_E_CUDA, LSG_E_TIMEOUT, LSG_E_STATE = 0, -1, -2, -3, -4, -5, -6
C128, C64 = 0, 1
R64, R32 = 2, 3  # real registers: density matrices in Pauli-transfer form
RD = 4  # real register of double-float pairs (two FP32 words per coefficient)
ELEM_BYTES = {C128: 16, C64: 8, R64: 8, R32: 4, RD: 8}
OP_MATRIX, OP_DIAG, OP_PERM, OP_DEPOL, OP_SCALE = 0, 1, 2, 3, 4
MAX_OP_BITS = 8

#: numpy layout of ``lsg_op`` (56 bytes: 10 int32, 2 int64)
OP_DTYPE = np.dtype(
    [("kind", "<i4"), ("nbits", "<i4"), ("bits", "<i4", (MAX_OP_BITS,)), ("data", "<i8"), ("batch_stride", "<i8")],
    align=True,
)
assert OP_DTYPE.itemsize == 56


class SimulationError(RuntimeError):
    """The circuit can't be simulated as asked (too large, or the method doesn't fit it)."""


class EngineError(RuntimeError):
    """The engine library or the GPU failed."""


_P = C.c_void_p
_I32, _I64, _D = C.c_int32, C.c_int64, C.c_double
_PD = C.POINTER(C.c_double)
_PI32 = C.POINTER(C.c_int32)
_PI64 = C.POINTER(C.c_int64)
_PU8 = C.POINTER(C.c_uint8)
_PU64 = C.POINTER(C.c_uint64)

SIGNATURES: dict[str, tuple[Any, list[Any]]] = {
    "lsg_last_error": (C.c_char_p, []),
    "lsg_version": (C.c_int, []),
    "lsg_init": (C.c_int, [C.c_int]),
    "lsg_max_bits": (C.c_int, []),
    "lsg_mem_info": (C.c_int, [_PI64, _PI64]),
    "lsg_state_create": (C.c_int, [C.c_int, C.c_int, _I64, C.POINTER(_P)]),
    "lsg_state_free": (C.c_int, [_P]),
    "lsg_state_set_basis": (C.c_int, [_P, _I64]),
    "lsg_state_upload": (C.c_int, [_P, _PD, _I64]),
    "lsg_state_download": (C.c_int, [_P, _PD, _I64]),
    "lsg_state_bytes": (C.c_int, [_P, _PI64]),
    "lsg_state_to_complex": (C.c_int, [_P, _I64, _P]),
    "lsg_apply": (C.c_int, [_P, _P, _I32, _PD, _I64]),
    "lsg_probabilities": (C.c_int, [_P, C.c_int, _I64, _PD]),
    "lsg_sample": (C.c_int, [_P, C.c_int, _I64, _PI32, _I32, _PD, _I64, _I32, _PI32, _PI32, _PD, _PD, _PD, _PU8, _PU8, _PI64]),
    "lsg_expect_pauli": (C.c_int, [_P, C.c_int, _PU64, _PU64, _I32, _PD]),
    "lsg_outcome_probabilities": (C.c_int, [_P, C.c_int, _PI32, _I32, _I32, _PI32, _PD, _PD, _D, _PD]),
    "lsg_prob_one": (C.c_int, [_P, C.c_int, _I64, _PD]),
    "lsg_program_create": (C.c_int, [_P, _P, _I32, _PD, _I64, C.POINTER(_P)]),
    "lsg_program_run": (C.c_int, [_P, _P]),
    "lsg_program_run_timed": (C.c_int, [_P, _P, C.POINTER(C.c_float)]),
    "lsg_program_info": (C.c_int, [_P, _PI32, _PI64]),
    "lsg_program_specialized": (C.c_int, [_P]),
    "lsg_jit_wanted": (C.c_int, [C.c_int64]),
    "lsg_apply_from_basis": (C.c_int, [_P, _I64, _P, _I32, _PD, _I64]),
    "lsg_program_run_from_basis": (C.c_int, [_P, _P, _I64, C.POINTER(C.c_float)]),
    "lsg_program_basis_info": (C.c_int, [_P, _PI64, _PI64]),
    "lsg_programs_run_ragged": (C.c_int, [_I32, C.POINTER(_P), C.POINTER(_P), _PI64, C.POINTER(C.c_float)]),
    "lsg_program_set_data": (C.c_int, [_P, _P, _P, _I32, _PD, _I64]),
    "lsg_program_graph_run": (C.c_int, [_P, _P, _I64]),
    "lsg_program_free": (C.c_int, [_P]),
    "lsg_program_create_opts": (C.c_int, [_P, _P, _I32, _PD, _I64, _P, C.POINTER(_P)]),
    "lsg_program_pass_info": (C.c_int, [_P, _I32, _PI64, _PD, _PI32]),
    "lsg_plan": (C.c_int, [C.c_int, C.c_int, _P, _I32, _PI32]),
    "lsg_program_source": (C.c_int, [C.c_int, C.c_int, _I64, _P, _I32, _PD, _I64, C.c_int, C.c_char_p, _I64, _PI64]),
    "lsg_state_sync": (C.c_int, [_P]),
    "lsg_state_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "lsg_collapse": (C.c_int, [_P, C.c_int, C.c_int, _D, _I64]),
}

_lib: C.CDLL | None = None
_lock = threading.Lock()
_tls = threading.local()  # the CUDA current device is per thread: bind each thread once
_default_device = 0


def set_device(device: int) -> None:
    """The device new registers go to (one process drives one GPU; ranks pick theirs)."""
    global _default_device
    _default_device = int(device)
    _tls.device = None
    ensure_device(_default_device)


def library() -> C.CDLL:
    """The loaded engine library (loaded once)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise EngineError(
                    f"the GB300 engine library is not built ({LIB_PATH} is missing); "
                    "run `python -m lucivant_sim_gb300.build`"
                )
            lib = C.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def check(code: int) -> None:
    if code == LSG_OK:
        return
    msg = library().lsg_last_error().decode(errors="replace")
    if code == LSG_E_ARG:
        raise ValueError(msg)
    if code == LSG_E_CAPACITY:
        raise SimulationError(msg)
    if code == LSG_E_MEMORY:
        raise MemoryError(msg)
    raise EngineError(f"engine error {code}: {msg}")


def ensure_device(device: int | None = None) -> None:
    dev = _default_device if device is None else device
    if getattr(_tls, "device", None) != dev:
        check(library().lsg_init(dev))
        _tls.device = dev


def mem_info() -> tuple[int, int]:
    """(free, total) bytes of this thread's device."""
    ensure_device()
    f, t = C.c_int64(0), C.c_int64(0)
    check(library().lsg_mem_info(C.byref(f), C.byref(t)))
    return int(f.value), int(t.value)


def plan_passes(nbits: int, precision: int, ops: "OpList") -> int:
    """Fused passes the engine plans for ``ops`` (host only, no device)."""
    table, _ = ops.packed()
    out = C.c_int32(0)
    check(library().lsg_plan(nbits, precision, table.ctypes.data, len(table), C.byref(out)))
    return int(out.value)


def jit_wanted(bytes_per_run: int) -> bool:
    """Whether the library specializes a program whose run moves ``bytes_per_run`` bytes."""
    rc = library().lsg_jit_wanted(int(bytes_per_run))
    if rc < 0:
        check(rc)
    return rc == 1


def specialized_source(nbits: int, precision: int, batch: int, ops: "OpList", compile: bool = False) -> str:
    """The CUDA source of the passes a program of ``ops`` would be specialized to ("" when it
    would be interpreted); with ``compile`` also compiled with NVRTC (host only, no device)."""
    table, pool = ops.packed()
    n = C.c_int64(0)
    lib = library()
    args = (nbits, precision, batch, table.ctypes.data, len(table), ptr(pool, C.c_double), pool.size // 2)
    check(lib.lsg_program_source(*args, 0, None, 0, C.byref(n)))
    buf = C.create_string_buffer(int(n.value) + 1)
    check(lib.lsg_program_source(*args, int(compile), buf, len(buf), C.byref(n)))
    return buf.value.decode()


def ptr(a: np.ndarray, ctype: Any) -> Any:
    return a.ctypes.data_as(C.POINTER(ctype))


class OpList:
    """Operators for one ``lsg_apply`` call and their complex128 data pool."""

    def __init__(self) -> None:
        self.rows: list[tuple[int, int, tuple[int, ...], int, int]] = []
        self.chunks: list[np.ndarray] = []
        self.size = 0

    def _data(self, arr: np.ndarray) -> int:
        flat = np.ascontiguousarray(arr, dtype=np.complex128).reshape(-1)
        at = self.size
        self.chunks.append(flat)
        self.size += flat.size
        return at

    def add(self, kind: int, bits: tuple[int, ...] | list[int], data: np.ndarray, batch_stride: int = 0) -> None:
        self.rows.append((kind, len(bits), tuple(int(b) for b in bits), self._data(data), batch_stride))

    def add_batched(self, kind: int, bits: tuple[int, ...] | list[int], per_member: np.ndarray) -> None:
        """``per_member[b]`` is member b's data (all the same size)."""
        per = np.ascontiguousarray(per_member, dtype=np.complex128)
        stride = int(per[0].size)
        self.rows.append((kind, len(bits), tuple(int(b) for b in bits), self._data(per), stride))

    def __len__(self) -> int:
        return len(self.rows)

    def packed(self) -> tuple[np.ndarray, np.ndarray]:
        """(operator table, float64 view of the pool), built column by column and kept until the
        next ``add``."""
        cached = getattr(self, "_packed", None)
        if cached is not None and cached[0] == len(self.rows):
            return cached[1]
        n = len(self.rows)
        ops = np.zeros(n, dtype=OP_DTYPE)
        if n:
            kinds, nbs, bitss, datas, strides = zip(*self.rows)
            ops["kind"] = kinds
            ops["nbits"] = nbs
            ops["data"] = datas
            ops["batch_stride"] = strides
            bits = np.zeros((n, MAX_OP_BITS), dtype=np.int32)
            widths = np.asarray(nbs)
            for w in np.unique(widths):
                rows = np.flatnonzero(widths == w)
                if w:
                    bits[rows, :w] = np.asarray([bitss[i] for i in rows], dtype=np.int32).reshape(len(rows), w)
            ops["bits"] = bits
        pool = np.concatenate(self.chunks) if self.chunks else np.zeros(1, dtype=np.complex128)
        out = ops, np.ascontiguousarray(pool.view(np.float64))
        self._packed = (n, out)
        return out


class Register:
    """A device register of ``batch`` members of 2^nbits amplitudes."""

    def __init__(self, nbits: int, precision: int = C128, batch: int = 1, device: int | None = None) -> None:
        ensure_device(device)
        self.lib = library()
        self.nbits, self.precision, self.batch = nbits, precision, batch
        handle = C.c_void_p()
        check(self.lib.lsg_state_create(nbits, precision, batch, C.byref(handle)))
        self.handle = handle

    def free(self) -> None:
        if getattr(self, "handle", None):
            self.lib.lsg_state_free(self.handle)
            self.handle = None

    def __del__(self) -> None:
        try:
            self.free()
        except Exception:
            pass

    def __enter__(self) -> Register:
        return self

    def __exit__(self, *exc: Any) -> None:
        self.free()

    def set_basis(self, index: int = 0) -> None:
        check(self.lib.lsg_state_set_basis(self.handle, index))

    def apply(self, ops: OpList) -> None:
        if not len(ops):
            return
        table, pool = ops.packed()
        check(self.lib.lsg_apply(self.handle, table.ctypes.data, len(table), ptr(pool, C.c_double), pool.size // 2))

    def apply_from_basis(self, ops: OpList, index: int = 0) -> None:
        """Every member set to basis state ``index``, then ``ops`` applied, skipping tiles the
        operators have not reached yet (the same result as ``set_basis`` + ``apply``)."""
        table, pool = ops.packed()
        check(self.lib.lsg_apply_from_basis(self.handle, index, table.ctypes.data, len(table), ptr(pool, C.c_double),
                                            pool.size // 2))  # fmt: skip

    @property
    def real(self) -> bool:
        """A Pauli-transfer (real) density register."""
        return self.precision in (R64, R32, RD)

    def download(self) -> np.ndarray:
        """(batch, 2^nbits) complex128 amplitudes, or float64 coefficients of a real register."""
        out = np.empty(self.batch << self.nbits, dtype=np.float64 if self.real else np.complex128)
        check(self.lib.lsg_state_download(self.handle, ptr(out.view(np.float64), C.c_double), out.nbytes))
        return out.reshape(self.batch, -1)

    def upload(self, data: np.ndarray) -> None:
        a = np.ascontiguousarray(data, dtype=np.float64 if self.real else np.complex128).reshape(-1)
        check(self.lib.lsg_state_upload(self.handle, ptr(a.view(np.float64), C.c_double), a.nbytes))

    def to_complex(self, member: int, out: Register) -> None:
        """Member ``member`` of this real register into member 0 of complex register ``out``."""
        check(self.lib.lsg_state_to_complex(self.handle, member, out.handle))

    def probabilities(self, dm_qubits: int = 0, member: int = 0) -> np.ndarray:
        """One member's probabilities, or every member's (shape (batch, 2^n)) when member < 0."""
        n = dm_qubits if dm_qubits else self.nbits
        rows = self.batch if member < 0 else 1
        out = np.empty(rows << n, dtype=np.float64)
        check(self.lib.lsg_probabilities(self.handle, dm_qubits, member, ptr(out, C.c_double)))
        return out.reshape(self.batch, -1) if member < 0 else out

    def outcome_probabilities(self, dm_qubits: int, measured: list[int], pair_pos: list[int],
                              pair_err: list[tuple[float, float]], threshold: float) -> np.ndarray:  # fmt: skip
        """Probabilities of every combination of reported pair bits (index bit j = pair j), with
        each pair's readout flips applied on the device; member 0."""
        meas = np.asarray(measured, dtype=np.int32)
        pos = np.asarray(pair_pos, dtype=np.int32)
        p01 = np.asarray([e[0] for e in pair_err], dtype=np.float64)
        p10 = np.asarray([e[1] for e in pair_err], dtype=np.float64)
        out = np.empty(1 << len(pos), dtype=np.float64)
        check(self.lib.lsg_outcome_probabilities(self.handle, dm_qubits, ptr(meas, C.c_int32), len(meas), len(pos),
                                                 ptr(pos, C.c_int32), ptr(p01, C.c_double), ptr(p10, C.c_double),
                                                 float(threshold), ptr(out, C.c_double)))  # fmt: skip
        return out

    def sample(
        self,
        dm_qubits: int,
        measured: list[int],
        uniforms: np.ndarray,
        pair_pos: list[int],
        pair_err: list[tuple[float, float] | None],
        flip_uniforms: np.ndarray | None,
        member: int = 0,
    ) -> tuple[np.ndarray, np.ndarray, int]:
        shots = int(uniforms.size)
        npairs = len(pair_pos)
        meas = np.asarray(measured, dtype=np.int32)
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        pos = np.asarray(pair_pos, dtype=np.int32)
        has = np.asarray([e is not None for e in pair_err], dtype=np.int32)
        p01 = np.asarray([e[0] if e else 0.0 for e in pair_err], dtype=np.float64)
        p10 = np.asarray([e[1] if e else 0.0 for e in pair_err], dtype=np.float64)
        flips = np.ascontiguousarray(flip_uniforms if flip_uniforms is not None else np.zeros(1), dtype=np.float64)
        bits = np.zeros((max(shots, 1), max(npairs, 1)), dtype=np.uint8)
        near = np.zeros(max(shots, 1), dtype=np.uint8)
        count = C.c_int64(0)
        check(
            self.lib.lsg_sample(
                self.handle, dm_qubits, member, ptr(meas, C.c_int32), len(meas), ptr(u, C.c_double), shots, npairs,
                ptr(pos, C.c_int32), ptr(has, C.c_int32), ptr(p01, C.c_double), ptr(p10, C.c_double),
                ptr(flips, C.c_double), ptr(bits, C.c_uint8), ptr(near, C.c_uint8), C.byref(count),
            )
        )  # fmt: skip
        return bits[:shots, :npairs], near[:shots], int(count.value)

    def expect(self, dm_qubits: int, xmasks: list[int], zmasks: list[int]) -> np.ndarray:
        x = np.asarray(xmasks, dtype=np.uint64)
        z = np.asarray(zmasks, dtype=np.uint64)
        out = np.zeros((len(x), self.batch), dtype=np.float64)
        check(self.lib.lsg_expect_pauli(self.handle, dm_qubits, ptr(x, C.c_uint64), ptr(z, C.c_uint64), len(x),
                                        ptr(out, C.c_double)))  # fmt: skip
        return out

    def prob_one(self, qubit: int, member: int = 0) -> float:
        out = C.c_double(0.0)
        check(self.lib.lsg_prob_one(self.handle, qubit, member, C.byref(out)))
        return float(out.value)

    def collapse(self, qubit: int, outcome: int, probability: float, member: int = 0) -> None:
        check(self.lib.lsg_collapse(self.handle, qubit, outcome, probability, member))

    def sync(self) -> None:
        check(self.lib.lsg_state_sync(self.handle))

    def stream(self) -> int:
        """The register's CUDA stream handle (an integer cudaStream_t)."""
        out = C.c_void_p()
        check(self.lib.lsg_state_stream(self.handle, C.byref(out)))
        return int(out.value or 0)

    def device_bytes(self) -> int:
        out = C.c_int64(0)
        check(self.lib.lsg_state_bytes(self.handle, C.byref(out)))
        return int(out.value)


class _PlanOptsC(C.Structure):
    _fields_ = [("tile_bits", C.c_int32), ("low_bits", C.c_int32), ("ctas", C.c_int32), ("max_ops", C.c_int32)]


class PlanOpts:
    """Plan and launch choices of a program (``lsg_plan_opts``; 0 keeps a field's default)."""

    def __init__(self, tile_bits: int = 0, low_bits: int = 0, ctas: int = 0, max_ops: int = 0) -> None:
        self.tile_bits, self.low_bits, self.ctas, self.max_ops = int(tile_bits), int(low_bits), int(ctas), int(max_ops)

    def struct(self) -> _PlanOptsC:
        return _PlanOptsC(self.tile_bits, self.low_bits, self.ctas, self.max_ops)

    def as_dict(self) -> dict[str, int]:
        return {"tile_bits": self.tile_bits, "low_bits": self.low_bits, "ctas": self.ctas, "max_ops": self.max_ops}

    def __eq__(self, other: object) -> bool:
        return isinstance(other, PlanOpts) and self.as_dict() == other.as_dict()

    def __repr__(self) -> str:
        return f"PlanOpts({', '.join(f'{k}={v}' for k, v in self.as_dict().items())})"


def run_ragged(pairs: list[tuple[Program, Register]], index: list[int] | None = None,
               timed: bool = False, sync: bool = True) -> np.ndarray | None:
    """Run every (program, register) pair from a basis state (``Program.run_from_basis``) as one
    sequence of launches: launch k carries pass k of every program that has one, whatever the
    registers' widths and batches (one precision). ``timed``: wait and return each launch's device
    time in ms. ``sync``: wait for the registers and report device errors."""
    if not pairs:
        return None
    lib = library()
    n = len(pairs)
    progs = (C.c_void_p * n)(*[p.handle for p, _ in pairs])
    regs = (C.c_void_p * n)(*[r.handle for _, r in pairs])
    idx = np.zeros(n, dtype=np.int64) if index is None else np.ascontiguousarray(index, dtype=np.int64)
    if idx.shape != (n,):
        raise ValueError("one basis index per pair")
    steps = max(p.passes for p, _ in pairs)
    out = np.zeros(max(steps, 1), dtype=np.float32) if timed else None
    check(lib.lsg_programs_run_ragged(n, progs, regs, ptr(idx, C.c_int64), ptr(out, C.c_float) if timed else None))
    if sync:
        for _, r in pairs:
            r.sync()
    return out[:steps] if timed else None


class Program:
    """A planned, uploaded operator list for registers shaped like ``shape``: run it repeatedly
    without re-planning, re-uploading or synchronising."""

    def __init__(self, shape: Register, ops: OpList, opts: PlanOpts | None = None) -> None:
        self.lib = library()
        table, pool = ops.packed()
        handle = C.c_void_p()
        if opts is None:
            check(self.lib.lsg_program_create(shape.handle, table.ctypes.data, len(table), ptr(pool, C.c_double),
                                              pool.size // 2, C.byref(handle)))  # fmt: skip
        else:
            check(self.lib.lsg_program_create_opts(shape.handle, table.ctypes.data, len(table), ptr(pool, C.c_double),
                                                   pool.size // 2, C.byref(opts.struct()), C.byref(handle)))  # fmt: skip
        self.handle = handle
        self.opts = opts
        passes, nbytes = C.c_int32(0), C.c_int64(0)
        check(self.lib.lsg_program_info(handle, C.byref(passes), C.byref(nbytes)))
        self.passes, self.bytes_per_run = int(passes.value), int(nbytes.value)
        rc = self.lib.lsg_program_specialized(handle)
        if rc < 0:
            check(rc)
        self.specialized = rc == 1

    def run(self, reg: Register) -> None:
        check(self.lib.lsg_program_run(self.handle, reg.handle))

    def run_from_basis(self, reg: Register, index: int = 0, timed: bool = False) -> np.ndarray | None:
        """Set every member to basis state ``index`` and run, skipping tiles that are still zero
        (same result as ``reg.set_basis(index); self.run(reg)``). ``timed``: wait and return each
        pass's device time in ms."""
        if not timed:
            check(self.lib.lsg_program_run_from_basis(self.handle, reg.handle, index, None))
            return None
        out = np.zeros(max(self.passes, 1), dtype=np.float32)
        check(self.lib.lsg_program_run_from_basis(self.handle, reg.handle, index, ptr(out, C.c_float)))
        return out[: self.passes]

    @property
    def basis_bytes_per_run(self) -> int:
        """HBM bytes one :meth:`run_from_basis` moves (2 x tile bytes per tile visited)."""
        nbytes = C.c_int64(0)
        check(self.lib.lsg_program_basis_info(self.handle, C.byref(nbytes), None))
        return int(nbytes.value)

    def pass_info(self) -> dict[str, np.ndarray]:
        """Per pass: HBM bytes a run from a basis state moves (all tiles before the first such
        run), floating-point operations per register element, register blocks."""
        n = max(self.passes, 1)
        tiles = np.zeros(n, dtype=np.int64)
        flops = np.zeros(n, dtype=np.float64)
        blocks = np.zeros(n, dtype=np.int32)
        check(self.lib.lsg_program_pass_info(self.handle, n, ptr(tiles, C.c_int64), ptr(flops, C.c_double),
                                             ptr(blocks, C.c_int32)))  # fmt: skip
        k = self.passes
        return {"bytes": tiles[:k], "flops_per_element": flops[:k], "blocks": blocks[:k]}

    def set_data(self, reg: Register, ops: OpList) -> None:
        """Take the operator data of ``ops`` (the same template with other parameters) without
        planning or allocating again. :class:`EngineError` when ``ops`` plan differently (another
        structure). Ordered after ``reg``'s earlier work."""
        table, pool = ops.packed()
        check(self.lib.lsg_program_set_data(self.handle, reg.handle, table.ctypes.data, len(table),
                                            ptr(pool, C.c_double), pool.size // 2))  # fmt: skip

    def graph_run(self, reg: Register, index: int = 0) -> None:
        """``run_from_basis`` as one CUDA graph launch (captured on the first call for this
        register and index). Does not wait."""
        check(self.lib.lsg_program_graph_run(self.handle, reg.handle, index))

    def run_timed(self, reg: Register) -> np.ndarray:
        out = np.zeros(max(self.passes, 1), dtype=np.float32)
        check(self.lib.lsg_program_run_timed(self.handle, reg.handle, ptr(out, C.c_float)))
        return out[: self.passes]

    def free(self) -> None:
        if getattr(self, "handle", None):
            self.lib.lsg_program_free(self.handle)
            self.handle = None

    def __del__(self) -> None:
        try:
            self.free()
        except Exception:
            pass
