"""Build the engine library ``liblsg.so`` in-tree for sm_103a with nvcc.

Each ``csrc/*.cu`` compiles to an object in ``_build/`` (in parallel), then they link into
``lucivant_sim_gb300/liblsg.so``. Objects are rebuilt only when a source or header is newer.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "liblsg.so"
INCLUDE = PKG.parent / "include"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    found = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(found).exists():
        raise RuntimeError("nvcc not found: the engine library needs the CUDA toolkit to build")
    return found


def _headers_mtime() -> float:
    heads = list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return max((h.stat().st_mtime for h in heads), default=0.0)


# Device headers the run-time specializer (csrc/jit.cu) hands to NVRTC, by include name.
JIT_HEADERS = [("tile.cuh", CSRC / "tile.cuh"), ("common.cuh", CSRC / "common.cuh"),
               ("program.cuh", CSRC / "program.cuh"), ("../../include/lsg.h", INCLUDE / "lsg.h")]
# NVRTC has no C library: the fixed-width integer types the headers use
RTC_STDINT = """#pragma once
typedef signed char int8_t; typedef short int16_t; typedef int int32_t; typedef long long int64_t;
typedef unsigned char uint8_t; typedef unsigned short uint16_t; typedef unsigned int uint32_t;
typedef unsigned long long uint64_t; typedef unsigned long long uintptr_t;
typedef decltype(sizeof(0)) size_t;
"""


def _jit_headers() -> Path:
    """Write the headers as C string literals for csrc/jit.cu (rebuilt when a header changes)."""
    out = BUILD / "jit_headers.inc"
    if out.exists() and out.stat().st_mtime >= _headers_mtime():
        return out
    names = [n for n, _ in JIT_HEADERS] + ["stdint.h"]
    texts = [p.read_text() for _, p in JIT_HEADERS] + [RTC_STDINT]
    lines = ["// generated by build.py from the device headers: do not edit",
             f"static const int kJitHeaderCount = {len(names)};",
             "static const char* const kJitHeaderNames[] = {" + ", ".join(f'"{n}"' for n in names) + "};",
             "static const char* const kJitHeaderSources[] = {"]
    for t in texts:
        assert ')LSGJIT"' not in t
        lines.append(f'R"LSGJIT({t})LSGJIT",')
    lines.append("};")
    out.write_text("\n".join(lines) + "\n")
    return out


def _compile(src: Path, extra: list[str]) -> Path:
    obj = BUILD / (src.stem + ".o")
    if obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, _headers_mtime()):
        return obj
    cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-I", str(INCLUDE), "-I", str(BUILD), "-c", str(src), "-o", str(obj)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{proc.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile every CUDA source and link the shared library; returns its path."""
    BUILD.mkdir(exist_ok=True)
    _jit_headers()
    sources = sorted(CSRC.glob("*.cu"))
    with ThreadPoolExecutor(max_workers=max(1, min(len(sources), os.cpu_count() or 4))) as pool:
        objs = list(pool.map(lambda s: _compile(s, extra or []), sources))
    newest = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart", "-ldl"]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"linking liblsg.so failed:\n{proc.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
