"""Autotuner: a program's plan and launch choices picked by timing them on the device.

Orrery chooses its kernels by fixed thresholds (``engines.py:20-27``: the slice kernel from 2^14 or
2^18 entries, the batched product from inner blocks of 8 entries). Here the choices are searched
per program shape instead. A shape is the register (bits, precision, batch members) and the
structure of its operator list (kinds, bits, which operators carry per-member data), not the
operators' values. For each candidate:

* tile bits (the register bits a CTA holds in shared memory: the default 32 KB tile and the next
  larger one; smaller tiles were slower on every workload measured),
* CTAs per SM the specialized passes are compiled for (the default and one neighbour),

the program is planned, compiled and run from the basis state on the register itself, timed with
CUDA events per pass (once for programs of 200 ms or more, else the best of four runs); the fastest candidate is kept in memory for the process and in a JSON
file (``LSG_TUNE_CACHE``, default ``~/.cache/lucivant_sim_gb300/tune.json``) for later processes.
Every candidate applies the same operators in circuit order wherever they act on the same
elements; only the grouping of commuting operators into passes differs, so results agree within
the engine's tolerances (1e-12 for FP64 registers), checked by the GPU tests.
"""

from __future__ import annotations

import hashlib
import json
import os
import threading
from pathlib import Path
from typing import Any

import numpy as np

from lucivant_sim_gb300 import _lib

_DEFAULT_TILE = {16: 11, 8: 12, 4: 13}
_DEFAULT_CTAS = {_lib.C128: 1, _lib.R64: 1, _lib.C64: 2, _lib.R32: 3, _lib.RD: 2}
_lock = threading.Lock()
_memory: dict[str, dict[str, Any]] = {}


def cache_path() -> Path:
    env = os.environ.get("LSG_TUNE_CACHE")
    return Path(env) if env else Path.home() / ".cache" / "lucivant_sim_gb300" / "tune.json"


_identity: str | None = None


def engine_identity() -> str:
    """The build and device a timing belongs to: the engine library's contents, its ABI version
    and the device's memory size. A choice timed with another build or on another GPU model is
    searched again rather than reused."""
    global _identity
    if _identity is None:
        h = hashlib.sha256()
        try:
            h.update(_lib.LIB_PATH.read_bytes())
        except OSError:
            pass
        h.update(f"{_lib.library().lsg_version()}:{_lib.mem_info()[1]}".encode())
        _identity = h.hexdigest()[:16]
    return _identity


def shape_key(reg: _lib.Register, ops: _lib.OpList) -> str:
    """The program shape a choice is kept for: register and operator structure, not values, on
    this engine build and device (``engine_identity``)."""
    h = hashlib.sha256()
    h.update(f"{engine_identity()}:{reg.nbits}:{reg.precision}:{reg.batch}:".encode())
    for kind, nb, bits, _at, stride in ops.rows:
        h.update(f"{kind},{nb},{bits},{int(stride > 0)};".encode())
    return h.hexdigest()[:32]


def candidates(nbits: int, precision: int) -> list[_lib.PlanOpts]:
    """The search space for a register of ``nbits`` bits: tile bits around the default, CTAs per
    SM around the default; the default comes first."""
    eb = _lib.ELEM_BYTES[precision]
    k0 = min(_DEFAULT_TILE[eb], nbits)
    c0 = _DEFAULT_CTAS[precision]
    eb_log = {16: 4, 8: 3, 4: 2}[eb]
    tiles = [k for k in (k0, k0 + 1) if 5 <= k <= nbits and k + eb_log <= 16]
    ctas = [c0, c0 + 1 if c0 == 1 else c0 - 1]
    out = []
    for k in tiles:
        for c in ctas:
            out.append(_lib.PlanOpts(tile_bits=k, ctas=c))
    return out


def _load() -> dict[str, dict[str, Any]]:
    try:
        return json.loads(cache_path().read_text())
    except (OSError, ValueError):
        return {}


def _save(key: str, entry: dict[str, Any]) -> None:
    path = cache_path()
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        data = _load()
        data[key] = entry
        tmp = path.with_suffix(f".{os.getpid()}.tmp")  # concurrent processes never share one
        tmp.write_text(json.dumps(data, indent=1, sort_keys=True))
        tmp.replace(path)
    except OSError:
        pass  # a read-only home: the choice stays in memory for this process


def tuned_program(reg: _lib.Register, ops: _lib.OpList, search: bool = True) -> tuple[_lib.Program, dict[str, Any]]:
    """A program for ``ops`` on registers shaped like ``reg`` with the fastest known choices.

    An unknown shape is searched (when ``search``) on ``reg`` itself: its contents are replaced
    (every run starts from the basis state). Returns the program and the record of the choice
    (``opts``, per-candidate milliseconds, whether it came from the cache)."""
    key = shape_key(reg, ops)
    with _lock:
        entry = _memory.get(key)
        if entry is None:
            entry = _load().get(key)
            if entry is not None:
                _memory[key] = entry
    if entry is not None:
        opts = _lib.PlanOpts(**entry["opts"])
        try:
            return _lib.Program(reg, ops, opts), dict(entry, cached=True)
        except (ValueError, _lib.EngineError):  # a choice this build no longer plans: search again
            with _lock:
                _memory.pop(key, None)
    if not search:
        return _lib.Program(reg, ops), {"opts": None, "cached": False, "searched": False}
    timings: list[dict[str, Any]] = []
    best: tuple[float, _lib.PlanOpts] | None = None
    for opts in candidates(reg.nbits, reg.precision):
        try:
            prog = _lib.Program(reg, ops, opts)
        except (ValueError, _lib.EngineError) as exc:  # a plan that does not fit: skipped
            timings.append({"opts": opts.as_dict(), "error": str(exc)[:120]})
            continue
        try:
            ms = float(np.sum(prog.run_from_basis(reg, 0, timed=True)))
            if ms < 200.0:  # short programs: the best of a few more runs (first launches load modules)
                ms = min([ms] + [float(np.sum(prog.run_from_basis(reg, 0, timed=True))) for _ in range(3)])
        finally:
            prog.free()
        timings.append({"opts": opts.as_dict(), "ms": ms, "passes": prog.passes, "specialized": prog.specialized})
        if best is None or ms < best[0]:
            best = (ms, opts)
    if best is None:
        return _lib.Program(reg, ops), {"opts": None, "cached": False, "searched": True, "candidates": timings}
    entry = {"opts": best[1].as_dict(), "ms": best[0], "candidates": timings}
    with _lock:
        _memory[key] = entry
    _save(key, entry)
    return _lib.Program(reg, ops, best[1]), dict(entry, cached=False)


def wanted(explicit: bool | None) -> bool:
    """Whether to tune: ``explicit`` when given, else ``LSG_AUTOTUNE=1``."""
    if explicit is not None:
        return explicit
    return os.environ.get("LSG_AUTOTUNE", "0") == "1"
