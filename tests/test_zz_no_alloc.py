"""The allocation-free expectation entry point (``lsg_expect_pauli_noalloc``) gives the same
results as ``lsg_expect_pauli``.

It serves callers that own all device memory themselves — a runtime or framework with its own
memory pool and a hard budget, or a latency-bound loop that cannot pay for cudaMalloc/cudaFree's
device-wide synchronisation — so here the test allocates the amplitudes and the output buffer
(with torch) and passes their device pointers through the C ABI. The file sorts last so that a
run stopping at the first failure has already run every other test.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from lucivant_sim_gb300 import _lib, engine, qasm, workloads as wl

pytestmark = pytest.mark.gpu

ATOL = 1e-12  # complex128 path: same tolerance as the other expectation tests
ATOL_C64 = 1e-5  # complex64 amplitudes, FP64 accumulation


def _numpy_expect(vec: np.ndarray, xs: list[int], zs: list[int]) -> np.ndarray:
    """<v|P|v> per term, computed on the host from the amplitudes (independent of the library)."""
    idx = np.arange(vec.size, dtype=np.uint64)
    out = []
    for x, z in zip(xs, zs, strict=True):
        ny = bin(x & z).count("1") & 3
        w = np.conj(vec[idx ^ np.uint64(x)]) * vec
        masked, parity = idx & np.uint64(z), np.zeros_like(idx)
        while masked.any():
            parity ^= masked & np.uint64(1)
            masked >>= np.uint64(1)
        sign = 1.0 - 2.0 * parity.astype(np.float64)
        out.append(float(np.real((1j**ny) * np.sum(w * sign))))
    return np.array(out)


def _noalloc(lib, amps, precision, nbits, batch, dm, xs, zs, out, stream):
    fn = lib.lsg_expect_pauli_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int64, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                   C.c_int32, C.c_void_p, C.c_void_p]  # fmt: skip
    x = np.asarray(xs, dtype=np.uint64)
    z = np.asarray(zs, dtype=np.uint64)
    return fn(amps, precision, nbits, batch, dm, x.ctypes.data_as(C.POINTER(C.c_uint64)),
              z.ctypes.data_as(C.POINTER(C.c_uint64)), len(x), out, stream)  # fmt: skip


def _terms(n: int, seed: int, count: int) -> tuple[list[int], list[int]]:
    masks = [engine.pauli_masks(lab) for lab in wl.random_pauli_sum(n, count, seed)]
    return [m[0] for m in masks], [m[1] for m in masks]


def test_noalloc_matches_expect_pauli_twice_in_a_row():
    torch = pytest.importorskip("torch")
    lib = _lib.library()
    n, batch = 10, 3
    circuit = qasm.parse(wl.hea(n, 3, seed=4))
    with _lib.Register(n, _lib.C128, batch=batch) as reg:
        reg.apply(engine.sv_oplist(circuit))
        host = reg.download()
        amps = torch.from_numpy(host.reshape(-1).copy()).to("cuda")
        stream = torch.cuda.current_stream().cuda_stream
        for seed, count in ((1, 7), (2, 12)):  # two calls in a row share the scratch array
            xs, zs = _terms(n, seed, count)
            want = reg.expect(0, xs, zs)
            out = torch.full((count * batch,), float("nan"), dtype=torch.float64, device="cuda")
            rc = _noalloc(lib, amps.data_ptr(), _lib.C128, n, batch, 0, xs, zs, out.data_ptr(), stream)
            assert rc == 0, lib.lsg_last_error().decode()
            got = out.cpu().numpy().reshape(count, batch)
            assert np.max(np.abs(got - want)) < ATOL
            for b in range(batch):  # and against a host computation from the same amplitudes
                assert np.max(np.abs(got[:, b] - _numpy_expect(host[b].reshape(-1), xs, zs))) < ATOL


def test_noalloc_complex64_matches_expect_pauli_and_refuses_bad_requests():
    torch = pytest.importorskip("torch")
    lib = _lib.library()
    n, batch = 9, 2
    circuit = qasm.parse(wl.hea(n, 2, seed=6))
    with _lib.Register(n, _lib.C64, batch=batch) as reg:
        reg.apply(engine.sv_oplist(circuit))
        host = reg.download()  # complex128 on the host: the device holds complex64
        amps = torch.from_numpy(host.reshape(-1).astype(np.complex64)).to("cuda")
        stream = torch.cuda.current_stream().cuda_stream
        xs, zs = _terms(n, 3, 10)
        want = reg.expect(0, xs, zs)
        out = torch.full((10 * batch,), float("nan"), dtype=torch.float64, device="cuda")
        for _ in range(2):  # two calls in a row
            rc = _noalloc(lib, amps.data_ptr(), _lib.C64, n, batch, 0, xs, zs, out.data_ptr(), stream)
            assert rc == 0, lib.lsg_last_error().decode()
            got = out.cpu().numpy().reshape(10, batch)
            assert np.max(np.abs(got - want)) < ATOL_C64
            exact = _numpy_expect(host[0].reshape(-1).astype(np.complex128), xs, zs)
            assert np.max(np.abs(got[:, 0] - exact)) < ATOL_C64
        # a host buffer is not device memory: refused before any launch
        host_out = np.zeros(10 * batch)
        rc = _noalloc(lib, amps.data_ptr(), _lib.C64, n, batch, 0, xs, zs, host_out.ctypes.data, stream)
        assert rc == _lib.LSG_E_ARG and b"device memory" in lib.lsg_last_error()
    # more members than one launch's grid takes: refused with a message, not a launch failure
    members = 65_536
    many = torch.zeros(members, dtype=torch.complex64, device="cuda")  # one amplitude per member
    out = torch.zeros(members, dtype=torch.float64, device="cuda")
    rc = _noalloc(lib, many.data_ptr(), _lib.C64, 0, members, 0, [0], [0], out.data_ptr(), stream)
    assert rc == _lib.LSG_E_ARG and b"at most 65535" in lib.lsg_last_error()


def test_noalloc_density_register_and_size_limit():
    torch = pytest.importorskip("torch")
    lib = _lib.library()
    n = 4
    circuit = qasm.parse(wl.brickwork(n, 2, seed=3, measure=False))
    with _lib.Register(2 * n, _lib.C128, batch=1) as reg:
        reg.apply(engine.dm_oplist(circuit, [wl.dm_noise()]))
        amps = torch.from_numpy(reg.download().reshape(-1).copy()).to("cuda")
        xs, zs = _terms(n, 5, 9)
        want = reg.expect(n, xs, zs)
        out = torch.zeros(9, dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        rc = _noalloc(lib, amps.data_ptr(), _lib.C128, 2 * n, 1, n, xs, zs, out.data_ptr(), stream)
        assert rc == 0, lib.lsg_last_error().decode()
        assert np.max(np.abs(out.cpu().numpy().reshape(9, 1) - want)) < ATOL
        # a request whose partial sums cannot fit the fixed scratch array is refused, not truncated
        many = 200_000
        big = torch.zeros(many, dtype=torch.float64, device="cuda")
        rc = _noalloc(lib, amps.data_ptr(), _lib.C128, 2 * n, 1, n, [0] * many, [1] * many, big.data_ptr(), stream)
        assert rc == _lib.LSG_E_ARG and b"scratch array" in lib.lsg_last_error()
