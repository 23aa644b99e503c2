"""The ctypes bindings agree with the C prototypes of ``include/lsg.h`` (no GPU needed).

A binding whose argument count or integer widths differ from the prototype still loads and may
even run, passing truncated or garbage upper bits; so every binding the package declares
(``_lib.SIGNATURES``, the stabilizer, trajectory and per-shot bindings) is compared here with
the header, argument by argument: integers by width and signedness, floating-point types
exactly, pointers by what they point to where the binding says so.
"""

from __future__ import annotations

import ctypes as C
import re
from pathlib import Path
from types import SimpleNamespace

import pytest

from lucivant_sim_gb300 import _lib, stabilizer, stabilizer_shots, trajectories

HEADER = Path(__file__).resolve().parents[1] / "include" / "lsg.h"
HANDLES = {"lsg_state", "lsg_program", "lsg_traj", "lsg_tab"}
SCALARS = {
    "int": C.c_int, "int32_t": C.c_int32, "int64_t": C.c_int64, "uint64_t": C.c_uint64,
    "int16_t": C.c_int16, "uint8_t": C.c_uint8, "double": C.c_double, "float": C.c_float,
}  # fmt: skip


def prototypes() -> dict[str, tuple[str, list[str]]]:
    text = re.sub(r"/\*.*?\*/", " ", HEADER.read_text(), flags=re.S)
    text = re.sub(r"^\s*#.*$", " ", text, flags=re.M)
    out = {}
    for ret, name, params in re.findall(r"([A-Za-z_][\w\s\*]*?)\b(lsg_\w+)\s*\(([^)]*)\)\s*;", text):
        ret = " ".join(ret.split()[-2:]) if "char" in ret else ret.split()[-1]
        args = [] if params.strip() in ("", "void") else [" ".join(p.split()) for p in params.split(",")]
        out[name] = (ret.strip(), args)
    return out


def c_type(param: str) -> tuple[str, int]:
    """(base type, pointer depth) of one parameter declaration, const and the name dropped."""
    p = param.replace("const ", "").strip()
    depth = p.count("*")
    p = p.replace("*", " ").split()
    base = p[0]
    if base in HANDLES:  # opaque handles are pointers
        depth += 1
        base = "void"
    return base, depth


def compatible(param: str, ct) -> bool:
    base, depth = c_type(param)
    if depth == 0:
        want = SCALARS[base]
        return C.sizeof(ct) == C.sizeof(want) and _kind(ct) == _kind(want)
    if ct in (C.c_void_p, C.c_char_p):
        return True
    target = getattr(ct, "_type_", None)
    if target is None:
        return False
    if depth >= 2 or (depth == 1 and base == "void" and param.split()[0] in HANDLES):
        return target in (C.c_void_p,) or getattr(target, "_type_", None) is not None
    if base in ("void", "char"):
        return True
    want = SCALARS[base]
    return C.sizeof(target) == C.sizeof(want) and _kind(target) == _kind(want)


def _kind(ct) -> str:
    if ct in (C.c_double, C.c_float):
        return "float"
    code = getattr(ct, "_type_", "")
    return "unsigned" if isinstance(code, str) and code.isupper() else "signed"


def bindings() -> dict[str, tuple[object, list]]:
    found = dict(_lib.SIGNATURES)
    found.update(stabilizer._SIGS)
    found.update(trajectories._SIGS)
    fake = SimpleNamespace(lsg_per_shot_run=SimpleNamespace())
    fn = stabilizer_shots._sig(fake)
    found["lsg_per_shot_run"] = (fn.restype, fn.argtypes)
    return found


def test_header_parses_every_declared_function():
    protos = prototypes()
    assert len(protos) >= 50
    assert protos["lsg_last_error"] == ("const char*", []) or protos["lsg_last_error"][0].endswith("char*")
    assert protos["lsg_apply"][1][0].startswith("lsg_state")


@pytest.mark.parametrize("name", sorted(bindings()))
def test_binding_matches_prototype(name):
    protos = prototypes()
    assert name in protos, f"{name} is bound but not declared in include/lsg.h"
    ret, params = protos[name]
    res, args = bindings()[name]
    assert len(args) == len(params), f"{name}: {len(args)} ctypes arguments, {len(params)} in the prototype"
    for i, (param, ct) in enumerate(zip(params, args, strict=True)):
        assert compatible(param, ct), f"{name} argument {i}: prototype '{param}', binding {ct}"
    if "char" in ret:
        assert res in (C.c_char_p, C.c_void_p)
    else:
        assert res is not None and C.sizeof(res) == C.sizeof(SCALARS[ret]), f"{name}: return {ret}, binding {res}"


def test_every_declared_function_used_by_the_package_is_bound():
    """Each prototype has a binding in the package, except the allocation-free entry point, which
    its callers bind themselves (its test does)."""
    unbound = set(prototypes()) - set(bindings()) - {"lsg_expect_pauli_noalloc"}
    assert not unbound, sorted(unbound)
