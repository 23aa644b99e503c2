"""An OpenQASM 2 / 3 reader producing :class:`~lucivant_sim_gb300.circuit.Circuit`.

It accepts the same language as Orrery's reader (``src/lucivant_sim/qasm.py:1-9``): register
and ``qubit``/``bit`` declarations, the qelib1/stdgates gates, user ``gate`` definitions, the
``ctrl``/``negctrl``/``inv``/``pow`` modifiers, ``input`` and ``const`` values, broadcasting,
index sets and ranges, both ``measure`` spellings, ``reset``, ``barrier``, ``gphase``, ``box``,
``delay`` and ``if``/``else`` on classical bits. Unsupported statements are refused with the same
messages, and a gate's noise label is the modifiers followed by its canonical name
(``qasm.py:721``), so noise rules attach exactly as they do in Orrery.
"""

from __future__ import annotations

import math
import re
from collections.abc import Callable, Mapping
from dataclasses import dataclass, field
from pathlib import Path
from typing import Any, NamedTuple

import numpy as np

from lucivant_sim_gb300.circuit import (
    Barrier,
    Circuit,
    Condition,
    Gate,
    GlobalPhase,
    IfElse,
    Measure,
    Register,
    Reset,
)
from lucivant_sim_gb300.gates import GATES, Matrix, canonical_name, controlled, gate_matrix, matrix_power, negcontrolled

MAX_QUBITS = 2048


class QasmError(ValueError):
    """The program can't be read; ``line``/``column`` locate the problem (1-based, 0 = unknown)."""

    def __init__(self, message: str, line: int = 0, column: int = 0) -> None:
        self.line, self.column = line, column
        super().__init__(f"line {line}, column {column}: {message}" if line else message)


class Tok(NamedTuple):
    kind: str  # id num str op phys eof
    text: str
    line: int
    col: int


_LEX = re.compile(
    r"""(?P<nl>\n)|(?P<sp>[ \t\r\f\v]+)|(?P<lc>//[^\n]*)|(?P<bc>/\*.*?\*/)
    |(?P<num>0[bB][01_]+|0[xX][0-9a-fA-F_]+|0[oO][0-7_]+|(?:\d[\d_]*\.?[\d_]*|\.\d[\d_]*)(?:[eE][+-]?\d+)?)
    |(?P<str>"[^"\n]*"|'[^'\n]*')|(?P<phys>\$\d+)|(?P<id>[^\W\d]\w*)
    |(?P<op>->|==|!=|<=|>=|&&|\|\||\*\*|<<|>>|[\[\](){};,:=+\-*/^%<>!~@&|.])""",
    re.VERBOSE | re.DOTALL,
)
_PRAGMA = re.compile(r"(?m)^[ \t]*(#?pragma|@)[^\n]*")


def tokenize(text: str) -> list[Tok]:
    text = _PRAGMA.sub("", text)
    out: list[Tok] = []
    line, start, pos = 1, 0, 0
    while pos < len(text):
        m = _LEX.match(text, pos)
        if m is None:
            raise QasmError(f"unexpected character {text[pos]!r}", line, pos - start + 1)
        kind = m.lastgroup or ""
        if kind == "nl":
            line, start = line + 1, m.end()
        elif kind == "bc":
            chunk = m.group()
            if "\n" in chunk:
                line += chunk.count("\n")
                start = pos + chunk.rfind("\n") + 1
        elif kind not in ("sp", "lc"):
            out.append(Tok(kind, m.group(), line, pos - start + 1))
        pos = m.end()
    out.append(Tok("eof", "", line, pos - start + 1))
    return out


_CONST = {"pi": math.pi, "π": math.pi, "tau": math.tau, "τ": math.tau, "euler": math.e, "ℇ": math.e}
_FUNC: dict[str, Callable[[float], float]] = {
    "sin": math.sin, "cos": math.cos, "tan": math.tan, "arcsin": math.asin, "asin": math.asin,
    "arccos": math.acos, "acos": math.acos, "arctan": math.atan, "atan": math.atan, "exp": math.exp,
    "ln": math.log, "log": math.log, "sqrt": math.sqrt,
}  # fmt: skip
_STD_INCLUDES = {"qelib1.inc", "stdgates.inc"}
_UNSUPPORTED = ("for", "while", "def", "defcal", "cal", "extern", "opaque", "return", "break", "continue")

# qelib1.inc defines the relative-phase Toffolis by decomposition, not as matrices.
_PRELUDE = """
gate rccx a,b,c { u2(0,pi) c; u1(pi/4) c; cx b,c; u1(-pi/4) c; cx a,c; u1(pi/4) c; cx b,c;
  u1(-pi/4) c; u2(0,pi) c; }
gate rc3x a,b,c,d { u2(0,pi) d; u1(pi/4) d; cx c,d; u1(-pi/4) d; u2(0,pi) d; cx a,d; u1(pi/4) d;
  cx b,d; u1(-pi/4) d; cx a,d; u1(pi/4) d; cx b,d; u1(-pi/4) d; u2(0,pi) d; u1(pi/4) d; cx c,d;
  u1(-pi/4) d; u2(0,pi) d; }
"""


def _number(text: str) -> float:
    t = text.replace("_", "").lower()
    for prefix, base in (("0b", 2), ("0x", 16), ("0o", 8)):
        if t.startswith(prefix):
            return float(int(t[2:], base))
    return float(t)


def embed(op: Matrix, sub: Matrix, positions: tuple[int, ...], k: int) -> Matrix:
    """``sub`` acting on local qubits ``positions`` of a k-qubit operator, applied after ``op``."""
    m = len(positions)
    t = op.reshape([2] * k + [1 << k])
    t = np.tensordot(sub.reshape([2] * (2 * m)), t, axes=(list(range(m, 2 * m)), list(positions)))
    return np.moveaxis(t, list(range(m)), list(positions)).reshape(1 << k, 1 << k)


@dataclass
class _Call:
    mods: list[tuple[str, Any]]
    name: Tok
    params: list[Any]
    args: list[str]


@dataclass
class _Def:
    params: list[str]
    qubits: list[str]
    body: list[Any]  # _Call or ("gphase", expr)


@dataclass
class _Scope:
    qregs: dict[str, Register] = field(default_factory=dict)
    cregs: dict[str, Register] = field(default_factory=dict)
    values: dict[str, float] = field(default_factory=dict)
    nq: int = 0
    nc: int = 0
    physical: int = -1


class _Reader:
    def __init__(self, text: str, inputs: Mapping[str, float], include: Callable[[str], str] | None,
                 scope: _Scope | None = None, defs: dict[str, _Def] | None = None) -> None:  # fmt: skip
        self.toks = tokenize(text)
        self.i = 0
        self.inputs = dict(inputs)
        self.used: dict[str, float] = {}
        self.include = include
        self.scope = scope or _Scope()
        self.defs: dict[str, _Def] = {} if defs is None else defs
        if defs is None:
            prelude = _Reader(_PRELUDE, {}, None, self.scope, self.defs)
            while prelude.peek().kind != "eof":
                prelude.gate_def(user=False)
        self.user: set[str] = set()

    # tokens
    def peek(self, ahead: int = 0) -> Tok:
        return self.toks[min(self.i + ahead, len(self.toks) - 1)]

    def take(self) -> Tok:
        t = self.peek()
        self.i += 1
        return t

    def fail(self, msg: str, tok: Tok | None = None) -> QasmError:
        t = tok or self.peek()
        return QasmError(msg, t.line, t.col)

    def is_(self, text: str, ahead: int = 0) -> bool:
        t = self.peek(ahead)
        return t.text == text and t.kind in ("op", "id")

    def accept(self, text: str) -> bool:
        if self.is_(text):
            self.i += 1
            return True
        return False

    def expect(self, text: str) -> Tok:
        t = self.peek()
        if not self.is_(text):
            found = "the end of the program" if t.kind == "eof" else repr(t.text)
            raise self.fail(f"expected {text!r} but found {found}", t)
        self.i += 1
        return t

    def name(self) -> Tok:
        t = self.take()
        if t.kind != "id":
            raise self.fail(f"expected a name but found {t.text!r}", t)
        return t

    # expressions: trees of tuples, evaluated late so gate bodies can bind parameters
    def expr(self) -> Any:
        node = self.term()
        while self.peek().kind == "op" and self.peek().text in ("+", "-"):
            node = ("bin", self.take().text, node, self.term())
        return node

    def term(self) -> Any:
        node = self.unary()
        while self.peek().kind == "op" and self.peek().text in ("*", "/", "%"):
            node = ("bin", self.take().text, node, self.unary())
        return node

    def unary(self) -> Any:
        if self.peek().kind == "op" and self.peek().text in ("-", "+"):
            sign = self.take().text
            inner = self.unary()
            return ("neg", inner) if sign == "-" else inner
        base = self.atom()
        if self.peek().kind == "op" and self.peek().text in ("^", "**"):
            self.take()
            return ("bin", "**", base, self.unary())
        return base

    def atom(self) -> Any:
        t = self.take()
        if t.kind == "num":
            return ("num", _number(t.text))
        if t.kind == "op" and t.text == "(":
            inner = self.expr()
            self.expect(")")
            return inner
        if t.kind == "id":
            if t.text in _FUNC and self.is_("("):
                self.take()
                arg = self.expr()
                self.expect(")")
                return ("fn", t.text, arg, t)
            return ("var", t.text, t)
        raise self.fail(f"expected a number or an expression but found {t.text!r}", t)

    def value(self, node: Any, env: Mapping[str, float] | None = None) -> float:
        tag = node[0]
        if tag == "num":
            return node[1]
        if tag == "var":
            key = node[1]
            if env and key in env:
                return env[key]
            if key in self.scope.values:
                return self.scope.values[key]
            if key in _CONST:
                return _CONST[key]
            raise self.fail(f"unknown name {key!r}", node[2])
        if tag == "neg":
            return -self.value(node[1], env)
        if tag == "fn":
            try:
                return _FUNC[node[1]](self.value(node[2], env))
            except ValueError as exc:
                raise self.fail(f"{node[1]}: {exc}", node[3]) from exc
        a, b = self.value(node[2], env), self.value(node[3], env)
        try:
            return {
                "+": lambda: a + b, "-": lambda: a - b, "*": lambda: a * b, "/": lambda: a / b,
                "%": lambda: math.fmod(a, b), "**": lambda: float(a**b),
            }[node[1]]()  # fmt: skip
        except (ZeroDivisionError, OverflowError, TypeError) as exc:
            raise self.fail(f"can't evaluate the expression: {exc}") from exc

    def whole(self, node: Any, what: str) -> int:
        v = self.value(node)
        if not math.isfinite(v) or abs(v - round(v)) > 1e-9:
            raise self.fail(f"{what} must be a whole number")
        return round(v)

    # program
    def program(self) -> list[Any]:
        if self.is_("OPENQASM"):
            self.take()
            t = self.take()
            major = t.text.split(".")[0]
            if t.kind != "num" or major not in ("2", "3"):
                raise self.fail("only OpenQASM 2 and 3 are supported", t)
            self.expect(";")
        ops: list[Any] = []
        while self.peek().kind != "eof":
            ops += self.statement()
        return ops

    def block(self) -> list[Any]:
        if not self.accept("{"):
            return self.statement()
        ops: list[Any] = []
        while not self.accept("}"):
            if self.peek().kind == "eof":
                raise self.fail("this block is never closed with '}'")
            ops += self.statement()
        return ops

    def statement(self) -> list[Any]:
        t = self.peek()
        word = t.text if t.kind == "id" else None
        if t.kind == "op" and t.text == ";":
            self.take()
            return []
        if word == "include":
            return self.include_stmt()
        if word in ("qreg", "creg"):
            self.take()
            reg = self.name()
            self.expect("[")
            size = self.whole(self.expr(), "a register size")
            self.expect("]")
            self.expect(";")
            self.declare(reg, size, quantum=word == "qreg")
            return []
        if word in ("qubit", "bit"):
            self.take()
            size = 1
            if self.accept("["):
                size = self.whole(self.expr(), "a register size")
                self.expect("]")
            reg = self.name()
            self.declare(reg, size, quantum=word == "qubit")
            if word == "bit" and self.accept("="):
                self.expect("measure")
                qs = self.qubits()
                self.expect(";")
                return self.measure_into(qs, self.clbits_of(reg.text))
            self.expect(";")
            return []
        if word == "gate":
            self.gate_def(user=True)
            return []
        if word in ("input", "const", "float", "angle", "int", "uint", "bool"):
            self.classical()
            return []
        if word == "measure":
            self.take()
            qs = self.qubits()
            if self.accept("->"):
                cs = self.clbits()
                self.expect(";")
                return self.measure_into(qs, cs)
            self.expect(";")
            return [Measure(q, None) for q in qs[0]]
        if word == "reset":
            self.take()
            qs = self.qubits()
            self.expect(";")
            return [Reset(q) for q in qs[0]]
        if word == "barrier":
            self.take()
            listed: list[int] = []
            while not self.is_(";"):
                listed += self.qubits()[0]
                if not self.accept(","):
                    break
            self.expect(";")
            return [Barrier(tuple(listed) or tuple(range(self.scope.nq)))]
        if word == "if":
            return [self.if_stmt()]
        if word == "box":
            self.take()
            if self.accept("["):
                self.skip_to("]")
            return self.block()
        if word == "delay":
            self.take()
            self.expect("[")
            self.skip_to("]")
            while not self.is_(";"):
                self.take()
            self.expect(";")
            return []
        if word in _UNSUPPORTED:
            raise self.fail(f"'{word}' isn't supported by Lucivant Orrery yet; unroll it or define a gate instead")
        if word == "gphase":
            self.take()
            self.expect("(")
            angle = self.value(self.expr())
            self.expect(")")
            self.expect(";")
            return [GlobalPhase(angle)]
        if t.kind == "id" and self.peek(1).text in ("=", "[") and t.text in self.scope.cregs:
            cs = self.clbits()
            self.expect("=")
            if not self.accept("measure"):
                raise self.fail("only measurement results can be assigned to bits")
            qs = self.qubits()
            self.expect(";")
            return self.measure_into(qs, cs)
        if t.kind == "id":
            return self.gate_stmt()
        raise self.fail("unexpected end of program" if t.kind == "eof" else f"unexpected {t.text!r}")

    def include_stmt(self) -> list[Any]:
        self.take()
        f = self.take()
        if f.kind != "str":
            raise self.fail("include needs a file name in quotes", f)
        self.expect(";")
        fname = f.text[1:-1]
        if fname in _STD_INCLUDES:
            return []
        if self.include is None:
            raise self.fail(f"can't include {fname!r}: only qelib1.inc and stdgates.inc are built in", f)
        nested = _Reader(self.include(fname), self.inputs, self.include, self.scope, self.defs)
        nested.user = self.user
        ops = nested.program()
        self.used.update(nested.used)
        return ops

    def skip_to(self, closing: str) -> None:
        depth = 0
        while True:
            t = self.take()
            if t.kind == "eof":
                raise self.fail(f"expected {closing!r}")
            if t.text == "[":
                depth += 1
            elif t.text == closing:
                if depth == 0:
                    return
                depth -= 1

    def declare(self, reg: Tok, size: int, *, quantum: bool) -> None:
        s = self.scope
        if reg.text in s.qregs or reg.text in s.cregs or reg.text in s.values:
            raise self.fail(f"{reg.text!r} is already declared", reg)
        if size < 1:
            raise self.fail("a register needs at least one bit", reg)
        if quantum:
            if s.physical >= 0:
                raise self.fail("a program can't mix declared qubits with physical qubits ($n)", reg)
            if s.nq + size > MAX_QUBITS:
                raise self.fail(f"more than {MAX_QUBITS} qubits", reg)
            s.qregs[reg.text] = Register(reg.text, s.nq, size)
            s.nq += size
        else:
            s.cregs[reg.text] = Register(reg.text, s.nc, size)
            s.nc += size

    def classical(self) -> None:
        is_input = self.accept("input")
        self.accept("const")
        typ = self.name()
        if typ.text not in ("float", "angle", "int", "uint", "bool"):
            raise self.fail(f"'{typ.text}' parameters aren't supported; use float or angle", typ)
        if self.accept("["):
            self.skip_to("]")
        var = self.name()
        if var.text in self.scope.values:
            raise self.fail(f"{var.text!r} is already declared", var)
        if is_input:
            if var.text not in self.inputs:
                raise self.fail(f"the program needs a value for its input {var.text!r}", var)
            val = float(self.inputs[var.text])
            self.used[var.text] = val
        else:
            self.expect("=")
            val = self.value(self.expr())
        self.expect(";")
        self.scope.values[var.text] = val

    # operands
    def index_list(self, size: int, reg: Tok) -> list[int]:
        if self.accept("{"):
            picks = [self.whole(self.expr(), "an index")]
            while self.accept(","):
                picks.append(self.whole(self.expr(), "an index"))
            self.expect("}")
        else:
            first = self.whole(self.expr(), "an index")
            if self.accept(":"):
                second = self.whole(self.expr(), "an index")
                if self.accept(":"):
                    step, stop = second, self.whole(self.expr(), "an index")
                else:
                    step, stop = 1, second
                if step == 0:
                    raise self.fail("a range's step can't be 0", reg)
                picks = list(range(first, stop + (1 if step > 0 else -1), step))
            else:
                picks = [first]
        self.expect("]")
        out = []
        for i in picks:
            j = i + size if i < 0 else i
            if not 0 <= j < size:
                raise self.fail(f"index {i} is outside {reg.text!r}, which has {size}", reg)
            out.append(j)
        return out

    def qubits(self) -> tuple[list[int], bool]:
        t = self.take()
        s = self.scope
        if t.kind == "phys":
            if s.qregs:
                raise self.fail("a program can't mix declared qubits with physical qubits ($n)", t)
            n = int(t.text[1:])
            if n >= MAX_QUBITS:
                raise self.fail(f"more than {MAX_QUBITS} qubits", t)
            s.physical = max(s.physical, n)
            s.nq = s.physical + 1
            return [n], False
        if t.kind != "id":
            raise self.fail(f"expected a qubit but found {t.text!r}", t)
        reg = s.qregs.get(t.text)
        if reg is None:
            raise self.fail(f"unknown qubit register {t.text!r}", t)
        if self.accept("["):
            return [reg.offset + i for i in self.index_list(reg.size, t)], False
        return list(range(reg.offset, reg.offset + reg.size)), True

    def clbits(self) -> tuple[list[int], bool]:
        t = self.name()
        return self.clbits_of(t.text, t)

    def clbits_of(self, regname: str, tok: Tok | None = None) -> tuple[list[int], bool]:
        reg = self.scope.cregs.get(regname)
        if reg is None:
            raise self.fail(f"unknown classical register {regname!r}", tok)
        if tok is not None and self.accept("["):
            return [reg.offset + i for i in self.index_list(reg.size, tok)], False
        return list(range(reg.offset, reg.offset + reg.size)), True

    def measure_into(self, qs: tuple[list[int], bool], cs: tuple[list[int], bool]) -> list[Any]:
        if len(qs[0]) != len(cs[0]):
            raise self.fail(f"can't measure {len(qs[0])} qubits into {len(cs[0])} bits")
        return [Measure(q, c) for q, c in zip(qs[0], cs[0], strict=True)]

    def if_stmt(self) -> IfElse:
        self.expect("if")
        self.expect("(")
        negate = self.accept("!")
        reg = self.name()
        bits, _ = self.clbits_of(reg.text, reg)
        target = 1
        if self.peek().text in ("==", "!="):
            if self.take().text == "!=":
                negate = not negate
            rhs = self.take()
            if rhs.kind == "num":
                target = int(_number(rhs.text))
            elif rhs.text in ("true", "false"):
                target = int(rhs.text == "true")
            else:
                raise self.fail("a condition compares with a whole number", rhs)
        elif len(bits) != 1:
            raise self.fail("compare a register with a value, e.g. if (c == 1)", reg)
        self.expect(")")
        then = self.block()
        other = self.block() if self.accept("else") else []
        return IfElse(Condition(tuple(bits), target, negate), tuple(then), tuple(other))

    # gates
    def modifiers(self) -> list[tuple[str, Any]]:
        mods: list[tuple[str, Any]] = []
        while self.peek().kind == "id" and self.peek().text in ("ctrl", "negctrl", "inv", "pow"):
            ahead = 1
            if self.peek(1).text == "(":
                depth = 0
                while True:
                    t = self.peek(ahead)
                    if t.text == "(":
                        depth += 1
                    elif t.text == ")":
                        depth -= 1
                        if depth == 0:
                            break
                    elif t.kind == "eof":
                        break
                    ahead += 1
                ahead += 1
            if self.peek(ahead).text != "@":
                break
            word = self.take().text
            arg = None
            if self.accept("("):
                arg = self.expr()
                self.expect(")")
            self.expect("@")
            mods.append((word, arg))
        return mods

    def call_head(self) -> tuple[list[tuple[str, Any]], Tok, list[Any]]:
        mods = self.modifiers()
        gname = self.name()
        params: list[Any] = []
        if self.accept("(") and not self.accept(")"):
            params.append(self.expr())
            while self.accept(","):
                params.append(self.expr())
            self.expect(")")
        return mods, gname, params

    def gate_stmt(self) -> list[Any]:
        mods, gname, pexprs = self.call_head()
        params = tuple(self.value(p) for p in pexprs)
        operands: list[tuple[list[int], bool]] = []
        while not self.is_(";"):
            operands.append(self.qubits())
            if not self.accept(","):
                break
        self.expect(";")
        if gname.text == "gphase" and not operands:
            if len(params) != 1:
                raise self.fail("gphase takes one angle", gname)
            return [GlobalPhase(params[0])]
        matrix, arity = self.resolve(mods, gname, params)
        if len(operands) != arity:
            raise self.fail(f"{gname.text} acts on {arity} qubit(s) but was given {len(operands)}", gname)
        widths = {len(qs) for qs, whole_reg in operands if whole_reg or len(qs) > 1}
        if len(widths) > 1:
            raise self.fail("registers of different sizes can't be combined in one gate", gname)
        repeat = widths.pop() if widths else 1
        label = "".join(f"{m}@" for m, _ in mods) + canonical_name(gname.text)
        out: list[Any] = []
        for i in range(repeat):
            qs = tuple(q[i] if len(q) > 1 else q[0] for q, _ in operands)
            if len(set(qs)) != len(qs):
                raise self.fail(f"{gname.text} is given the same qubit twice", gname)
            out.append(Gate(label, qs, matrix, params))
        return out

    def resolve(self, mods: list[tuple[str, Any]], gname: Tok, params: tuple[float, ...],
                env: Mapping[str, float] | None = None) -> tuple[Matrix, int]:  # fmt: skip
        matrix, arity = self.base(gname, params)
        for word, arg in reversed(mods):
            if word == "inv":
                matrix = matrix.conj().T
            elif word == "pow":
                if arg is None:
                    raise self.fail("pow needs an exponent, e.g. pow(2) @", gname)
                matrix = matrix_power(matrix, self.value(arg, env))
            else:
                count = 1 if arg is None else self.whole(arg, "the number of controls")
                for _ in range(count):
                    matrix = controlled(matrix) if word == "ctrl" else negcontrolled(matrix)
                arity += count
        return matrix, arity

    def base(self, gname: Tok, params: tuple[float, ...]) -> tuple[Matrix, int]:
        d = self.defs.get(gname.text)
        if d is not None and (gname.text in self.user or gname.text not in GATES):
            if len(params) != len(d.params):
                raise self.fail(f"{gname.text} takes {len(d.params)} parameter(s) but was given {len(params)}", gname)
            return self.unitary(d, params), len(d.qubits)
        spec = GATES.get(gname.text)
        if spec is None:
            raise self.fail(f"unknown gate {gname.text!r}", gname)
        if len(params) != spec.params:
            raise self.fail(f"{gname.text} takes {spec.params} parameter(s) but was given {len(params)}", gname)
        return gate_matrix(gname.text, params), spec.qubits

    def unitary(self, d: _Def, params: tuple[float, ...]) -> Matrix:
        k = len(d.qubits)
        env = dict(zip(d.params, params, strict=True))
        where = {q: i for i, q in enumerate(d.qubits)}
        acc = np.eye(1 << k, dtype=np.complex128)
        for item in d.body:
            if isinstance(item, tuple):
                acc = acc * np.exp(1j * self.value(item[1], env))
                continue
            vals = tuple(self.value(p, env) for p in item.params)
            sub, arity = self.resolve(item.mods, item.name, vals, env)
            if len(item.args) != arity:
                raise self.fail(f"{item.name.text} acts on {arity} qubit(s) but was given {len(item.args)}", item.name)
            pos = tuple(where[a] for a in item.args)
            if len(set(pos)) != len(pos):
                raise self.fail(f"{item.name.text} is given the same qubit twice", item.name)
            acc = embed(acc, sub, pos, k)
        return acc

    def gate_def(self, *, user: bool) -> None:
        self.expect("gate")
        gname = self.name()
        if gname.text in self.user:
            raise self.fail(f"gate {gname.text!r} is already defined", gname)
        params: list[str] = []
        if self.accept("(") and not self.accept(")"):
            params.append(self.name().text)
            while self.accept(","):
                params.append(self.name().text)
            self.expect(")")
        qubits = [self.name().text]
        while self.accept(","):
            qubits.append(self.name().text)
        if len(set(qubits)) != len(qubits):
            raise self.fail("a gate's qubit arguments must have different names", gname)
        self.expect("{")
        body: list[Any] = []
        while not self.accept("}"):
            if self.peek().kind == "eof":
                raise self.fail(f"gate {gname.text!r} is never closed with '}}'", gname)
            if self.is_("barrier"):
                while self.take().text != ";":
                    pass
                continue
            mods, cname, cparams = self.call_head()
            if cname.text == "gphase":
                self.expect(";")
                if len(cparams) != 1:
                    raise self.fail("gphase takes one angle", cname)
                body.append(("gphase", cparams[0]))
                continue
            args: list[str] = []
            while not self.is_(";"):
                a = self.name()
                if a.text not in qubits:
                    raise self.fail(f"{a.text!r} isn't an argument of gate {gname.text!r}", a)
                args.append(a.text)
                if not self.accept(","):
                    break
            self.expect(";")
            if cname.text == gname.text:
                raise self.fail("a gate can't call itself", cname)
            body.append(_Call(mods, cname, cparams, args))
        self.defs[gname.text] = _Def(params, qubits, body)
        if user:
            self.user.add(gname.text)


# ---------------------------------------------------------------------------- plain programs
#
# Most programs a server or a benchmark sends are plain: declarations, standard gates with number
# or input arguments on indexed qubits, measurements. Those statements are read here by one regular
# expression each, without the token stream; anything else (comments, gate definitions,
# modifiers, expressions, broadcasting, ranges, conditions, resets, barriers, errors) sends the
# whole program to the general reader. Both produce the same Circuit, operation for operation.

_NUM = r"(?:\d[\d_]*\.?[\d_]*|\.\d[\d_]*)(?:[eE][+-]?\d+)?"
_FAST_ARG = re.compile(rf"\s*(-?)\s*(?:({_NUM})|([A-Za-z_]\w*))\s*$")
_FAST_GATE = re.compile(r"([A-Za-z_]\w*)\s*(?:\(([^()]*)\))?\s+(.+)", re.DOTALL)
_FAST_QARG = re.compile(r"\s*([A-Za-z_]\w*)\s*\[\s*(\d+)\s*\]\s*$")
_FAST_DECL = re.compile(r"(qubit|bit)\s*\[\s*(\d+)\s*\]\s*([A-Za-z_]\w*)$|(qreg|creg)\s+([A-Za-z_]\w*)\s*\[\s*(\d+)\s*\]$")
_FAST_MEASURE = re.compile(r"([A-Za-z_]\w*)\s*(?:\[\s*(\d+)\s*\])?\s*=\s*measure\s+([A-Za-z_]\w*)\s*(?:\[\s*(\d+)\s*\])?$")
_FAST_INPUT = re.compile(r"input\s+(?:float|angle)\s+([A-Za-z_]\w*)$")
_FAST_HEADER = re.compile(r"OPENQASM\s+[23](?:\.\d+)?$")
_FAST_INCLUDE = re.compile(r'include\s+"(?:stdgates\.inc|qelib1\.inc)"$')
_FAST_WORDS = frozenset(("OPENQASM", "include", "qubit", "bit", "qreg", "creg", "input", "measure", "reset",
                         "barrier", "if", "else", "gate", "gphase", "const", "box", "delay", "ctrl", "negctrl",
                         "inv", "pow", "float", "angle", "int", "uint", "bool"))  # fmt: skip


def _fast_parse(source: str, params: Mapping[str, float]) -> Circuit | None:
    """The Circuit of a plain program, or None when the general reader must read it."""
    # comments, blocks, modifiers, physical qubits, pragmas, strings other than two includes
    if any(c in source for c in "/{}@$#'\\") or source.count('"') > 4:
        return None
    stmts = source.split(";")
    if stmts[-1].strip():
        return None
    qregs: dict[str, Register] = {}
    cregs: dict[str, Register] = {}
    values: dict[str, float] = {}
    used: dict[str, float] = {}
    nq = nc = 0
    ops: list[Any] = []
    for k, raw in enumerate(stmts[:-1]):
        st = raw.strip()
        if not st:
            return None  # empty statements: the general reader keeps its own rules
        if k == 0 and st.startswith("OPENQASM"):
            if not _FAST_HEADER.match(st):
                return None
            continue
        if st.startswith("include"):
            if not _FAST_INCLUDE.match(st):
                return None
            continue
        m = _FAST_DECL.match(st)
        if m:
            quantum = (m.group(1) or m.group(4)) in ("qubit", "qreg")
            name = m.group(3) or m.group(5)
            size = int(m.group(2) or m.group(6))
            if size < 1 or name in qregs or name in cregs or name in values or name in _FAST_WORDS:
                return None
            if quantum:
                if nq + size > MAX_QUBITS:
                    return None
                qregs[name] = Register(name, nq, size)
                nq += size
            else:
                cregs[name] = Register(name, nc, size)
                nc += size
            continue
        m = _FAST_INPUT.match(st)
        if m:
            var = m.group(1)
            if var in values or var in qregs or var in cregs or var not in params:
                return None
            values[var] = used[var] = float(params[var])
            continue
        if "measure" in st:
            m = _FAST_MEASURE.match(st)
            if not m or m.group(1) not in cregs or m.group(3) not in qregs:
                return None
            creg, qreg = cregs[m.group(1)], qregs[m.group(3)]
            if (m.group(2) is None) != (m.group(4) is None):
                return None
            if m.group(2) is None:
                if creg.size != qreg.size:
                    return None
                ops += [Measure(qreg.offset + i, creg.offset + i) for i in range(qreg.size)]
            else:
                ci, qi = int(m.group(2)), int(m.group(4))
                if ci >= creg.size or qi >= qreg.size:
                    return None
                ops.append(Measure(qreg.offset + qi, creg.offset + ci))
            continue
        m = _FAST_GATE.match(st)
        if not m:
            return None
        gname, argtext, qtext = m.group(1), m.group(2), m.group(3)
        spec = GATES.get(gname)
        if spec is None or gname in _FAST_WORDS or gname in qregs or gname in cregs:
            return None
        vals: list[float] = []
        if argtext is not None and argtext.strip():
            for a in argtext.split(","):
                am = _FAST_ARG.match(a)
                if not am:
                    return None
                if am.group(2) is not None:
                    v = _number(am.group(2))
                elif am.group(3) in values:
                    v = values[am.group(3)]
                else:
                    return None  # constants and unknown names: the general reader
                vals.append(-v if am.group(1) else v)
        if len(vals) != spec.params:
            return None
        qs: list[int] = []
        for q in qtext.split(","):
            qm = _FAST_QARG.match(q)
            if not qm or qm.group(1) not in qregs:
                return None
            reg, i = qregs[qm.group(1)], int(qm.group(2))
            if i >= reg.size:
                return None
            qs.append(reg.offset + i)
        if len(qs) != spec.qubits or len(set(qs)) != len(qs):
            return None
        pv = tuple(vals)
        ops.append(Gate(canonical_name(gname), tuple(qs), gate_matrix(gname, pv), pv))
    if set(params) - set(used):
        return None
    return Circuit(nq, nc, tuple(ops), tuple(qregs.values()), tuple(cregs.values()), dict(used))


def parse(source: str, params: Mapping[str, float] | None = None, *, include_dir: str | Path | None = None) -> Circuit:
    """Read OpenQASM 2 or 3 source. ``params`` binds ``input`` values; ``include_dir`` allows
    includes of files inside that folder only."""
    include = None
    if include_dir is not None:
        root = Path(include_dir).resolve()

        def include(fname: str) -> str:
            path = (root / fname).resolve()
            if root not in path.parents:
                raise QasmError(f"include {fname!r} is outside {root}")
            return path.read_text(encoding="utf-8")

    if include_dir is None:
        plain = _fast_parse(source, params or {})
        if plain is not None:
            return plain
    reader = _Reader(source, params or {}, include)
    ops = reader.program()
    s = reader.scope
    qregs = tuple(s.qregs.values()) if s.physical < 0 else (Register("$", 0, s.nq),)
    extra = set(params or {}) - set(reader.used)
    if extra:
        raise QasmError(f"the program has no input named {', '.join(sorted(extra))}")
    return Circuit(s.nq, s.nc, tuple(ops), qregs, tuple(s.cregs.values()), dict(reader.used))


def load(path: str | Path, params: Mapping[str, float] | None = None) -> Circuit:
    p = Path(path)
    return parse(p.read_text(encoding="utf-8"), params, include_dir=p.parent)
