"""Record what Orrery's OpenQASM reader (lucivant-sim 0.3.0, ``qasm.parse``) makes of programs that
cover the language it reads and of malformed programs that reach each of its error messages, by
running Orrery itself.

Run from the repository root, in a checkout where Orrery's sources are readable:

    python tests/golden/make_golden_qasm.py /path/to/lucivant-sim/src

It writes ``tests/golden/qasm.json``: per program the source, the ``input`` values given, and
Orrery's answer: the circuit (digest, qubit and bit counts, registers, inputs, operation kinds,
whether it is dynamic, its final measurements, operation counts, bit-string formatting),
or the exception's class, message, line and column. The tests never need Orrery.
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

sys.dont_write_bytecode = True
HERE = Path(__file__).resolve().parent

V3 = 'OPENQASM 3.0;\ninclude "stdgates.inc";\n'
V2 = 'OPENQASM 2.0;\ninclude "qelib1.inc";\n'

# (name, source, input values)
VALID = [
    ("v2_basic", V2 + "qreg q[3]; creg c[3];\nu3(0.1,0.2,0.3) q[0]; u2(0.4,0.5) q[1]; u1(0.6) q[2];\n"
     "cx q[0],q[1]; barrier q; reset q[2]; measure q -> c;\n", {}),
    ("v2_if", V2 + "qreg q[2]; creg c[2];\nh q[0]; measure q[0] -> c[0];\nif (c == 1) x q[1];\nmeasure q[1] -> c[1];\n", {}),
    ("v3_stdgates", V3 + "qubit[4] q; bit[4] c;\nh q[0]; ry(0.3) q[1]; rz(-0.7) q[2]; crx(0.2) q[0], q[3];\n"
     "cp(pi/3) q[1], q[2]; swap q[2], q[3]; ccx q[0], q[1], q[2]; cswap q[3], q[0], q[1];\n"
     "sx q[0]; sdg q[1]; tdg q[2]; p(0.25) q[3]; cy q[0], q[2]; ch q[1], q[3];\nc = measure q;\n", {}),
    ("v3_partial_measure", V3 + "qubit[3] q; bit[2] c; bit[1] d;\nh q;\nc[0] = measure q[2];\nc[1] = measure q[0];\n"
     "d[0] = measure q[1];\n", {}),
    ("v3_gate_def", V3 + "gate mix(a, b) x, y { ry(a) x; cx x, y; rz(b * 2) y; }\n"
     "gate twice x { h x; h x; }\n"
     "qubit[2] q;\nmix(0.3, -0.4) q[0], q[1];\ntwice q[1];\n", {}),
    ("v3_modifiers", V3 + "qubit[3] q;\nctrl @ x q[0], q[1];\nnegctrl @ h q[1], q[2];\ninv @ s q[0];\n"
     "pow(2) @ sx q[1];\npow(0.5) @ z q[2];\nctrl(2) @ x q[0], q[1], q[2];\ninv @ pow(0.5) @ sx q[2];\n", {}),
    ("v3_inputs", V3 + "input float theta;\ninput angle phi;\nqubit[2] q;\nrx(theta) q[0];\nrz(phi / 2) q[1];\n",
     {"theta": 0.375, "phi": 1.25}),
    ("v3_physical", V3 + "h $0;\ncx $0, $2;\nbit[3] c;\nc[0] = measure $0;\nc[2] = measure $2;\n", {}),
    ("v3_ranges", V3 + "qubit[6] q;\nh q[0:2];\nx q[3:];\nz q[0:2:5];\ncx q[0:1], q[2:3];\nh q[-1];\n", {}),
    ("v3_ranges_ok", V3 + "qubit[6] q;\nh q[0:2];\nz q[0:2:5];\ncx q[0:1], q[2:3];\nh q[-1];\n", {}),
    ("v3_ifelse", V3 + "qubit[3] q; bit[3] c;\nh q[0];\nc[0] = measure q[0];\n"
     "if (c[0] == 1) { x q[1]; h q[2]; } else { h q[1]; }\nif (c == 1) z q[2];\nif (c[0]) x q[2];\n"
     "c = measure q;\n", {}),
    ("v3_expressions", V3 + "qubit q;\nrx(pi / 4 + 2 * 0.5 - -1) q;\nry(sin(0.3) ** 2 + cos(0.3) ^ 2) q;\n"
     "rz(sqrt(2) * exp(0.1) - ln(3)) q;\nU(tau / 8, 1.5e-1, -.5) q;\ngphase(pi / 2);\nrx(π / 8) q;\n"
     "rz(arctan(1) + arcsin(0.5) + arccos(0.2) + tan(0.1)) q;\n", {}),
    ("v3_comments", V3 + "// a line comment\nqubit[2] q; /* a block\ncomment */ bit[2] c;\nh q[0]; // trailing\n"
     "cx q[0], q[1];\nc = measure q;\n", {}),
    ("v3_delay_box", V3 + "qubit[2] q;\ndelay[100ns] q[0];\nbox { h q[0]; cx q[0], q[1]; }\nbarrier;\n", {}),
    ("v3_broadcast", V3 + "qubit[3] a; qubit[3] b; bit[3] c;\nh a;\ncx a, b;\nc = measure b;\n", {}),
    ("v3_old_measure", V3 + "qubit[2] q; bit[2] c;\nh q[0];\nmeasure q -> c;\nmeasure q[1] -> c[0];\n", {}),
    ("v3_old_decl", "OPENQASM 3;\ninclude \"stdgates.inc\";\nqreg q[2];\ncreg c[2];\nh q[0]; cx q[0], q[1];\n"
     "c = measure q;\n", {}),
    ("v3_reset_barrier", V3 + "qubit[3] q; bit[1] c;\nreset q;\nx q[1];\nbarrier q[0], q[1];\nreset q[1];\n"
     "c[0] = measure q[1];\n", {}),
    ("v3_gphase_in_gate", V3 + "gate ph(t) a { gphase(t); x a; }\nqubit q;\nph(0.5) q;\n", {}),
    ("v3_CX_U", V3 + "qubit[2] q;\nU(0.1, 0.2, 0.3) q[0];\nCX q[0], q[1];\n", {}),
    ("no_version", "include \"stdgates.inc\";\nqubit[2] q;\nh q[0];\ncx q[0], q[1];\n", {}),
    ("empty", "OPENQASM 3;\n", {}),
    ("v3_nested_if", V3 + "qubit[2] q; bit[2] c;\nc[0] = measure q[0];\nif (c[0] == 0) { if (c[1] == 0) { x q[1]; } }\n", {}),
    ("v3_rccx", V3 + "qubit[4] q;\nrccx q[0], q[1], q[2];\nrc3x q[0], q[1], q[2], q[3];\nc3x q[3], q[2], q[1], q[0];\n", {}),
]

INVALID = [
    ("bad_char", V3 + "qubit q;\nh q; @@\n", {}),
    ("missing_semicolon", V3 + "qubit q;\nh q\n", {}),
    ("expected_name", V3 + "qubit[2] 3;\n", {}),
    ("expected_expr", V3 + "qubit q;\nrx(*) q;\n", {}),
    ("unknown_name", V3 + "qubit q;\nrx(foo) q;\n", {}),
    ("math_error", V3 + "qubit q;\nrx(sqrt(-1)) q;\n", {}),
    ("div_zero", V3 + "qubit q;\nrx(1 / 0) q;\n", {}),
    ("not_whole", V3 + "qubit[2.5] q;\n", {}),
    ("version", "OPENQASM 4;\nqubit q;\n", {}),
    ("unclosed_block", V3 + "qubit q; bit c;\nc = measure q;\nif (c == 1) { x q;\n", {}),
    ("include_no_quotes", "OPENQASM 3;\ninclude stdgates.inc;\n", {}),
    ("include_other", "OPENQASM 3;\ninclude \"mygates.inc\";\n", {}),
    ("for_loop", V3 + "qubit q;\nfor int i in [0:2] { x q; }\n", {}),
    ("def_sub", V3 + "def f() { }\n", {}),
    ("assign_not_measure", V3 + "qubit q; bit c;\nc = 1;\n", {}),
    ("unexpected_token", V3 + "qubit q;\n) ;\n", {}),
    ("unexpected_end", V3 + "qubit q;\nrx(0.1\n", {}),
    ("expected_closing", V3 + "qubit q;\nrx(0.1 q;\n", {}),
    ("redeclared", V3 + "qubit q;\nqubit q;\n", {}),
    ("zero_register", V3 + "qubit[0] q;\n", {}),
    ("mix_physical", V3 + "qubit q;\nh $0;\n", {}),
    ("too_many_qubits", V3 + "qubit[3000] q;\n", {}),
    ("input_int", V3 + "input int n;\n", {}),
    ("input_redeclared", V3 + "input float a;\ninput float a;\n", {"a": 1.0}),
    ("input_missing", V3 + "input float theta;\nqubit q;\nrx(theta) q;\n", {}),
    ("input_unused", V3 + "qubit q;\nh q;\n", {"zz": 1.0}),
    ("range_step_zero", V3 + "qubit[3] q;\nh q[0:0:2];\n", {}),
    ("index_outside", V3 + "qubit[2] q;\nh q[5];\n", {}),
    ("expected_qubit", V3 + "qubit q;\nh 3;\n", {}),
    ("gate_unknown_arg", V3 + "gate g a { h b; }\n", {}),
    ("unknown_qreg", V3 + "qubit q;\nh r[0];\n", {}),
    ("unknown_creg", V3 + "qubit q;\nmeasure q -> d;\n", {}),
    ("measure_size", V3 + "qubit[2] q; bit[3] c;\nc = measure q;\n", {}),
    ("cond_not_whole", V3 + "qubit q; bit c;\nc = measure q;\nif (c == 1.5) x q;\n", {}),
    ("cond_no_value", V3 + "qubit q; bit[2] c;\nif (c) x q;\n", {}),
    ("gphase_two", V3 + "gphase(1, 2);\n", {}),
    ("arity", V3 + "qubit[2] q;\ncx q[0];\n", {}),
    ("register_sizes", V3 + "qubit[2] a; qubit[3] b;\ncx a, b;\n", {}),
    ("same_qubit", V3 + "qubit[2] q;\ncx q[0], q[0];\n", {}),
    ("pow_no_exponent", V3 + "qubit q;\npow @ x q;\n", {}),
    ("unknown_gate", V3 + "qubit q;\nfoo q;\n", {}),
    ("param_count", V3 + "qubit q;\nrx(0.1, 0.2) q;\n", {}),
    ("param_missing", V3 + "qubit q;\nrx q;\n", {}),
    ("def_arity", V3 + "gate g a, b { cx a; }\nqubit[2] q;\ng q[0], q[1];\n", {}),
    ("def_same_qubit", V3 + "gate g a, b { cx a, a; }\n", {}),
    ("def_same_qubit_call", V3 + "gate g a, b { cx a, a; }\nqubit[2] q;\ng q[0], q[1];\n", {}),
    ("def_not_argument_call", V3 + "gate g(t) a { rx(u) a; }\nqubit q;\ng(0.1) q;\n", {}),
    ("def_twice", V3 + "gate g a { h a; }\ngate g a { x a; }\n", {}),
    ("def_same_names", V3 + "gate g a, a { h a; }\n", {}),
    ("def_unclosed", V3 + "gate g a { h a;\n", {}),
    ("def_gphase_two", V3 + "gate g a { gphase(1, 2); }\n", {}),
    ("def_not_argument", V3 + "gate g(t) a { rx(u) a; }\n", {}),
    ("def_recursive", V3 + "gate g a { g a; }\n", {}),
    ("call_arity", V3 + "gate g a, b { cx a, b; }\nqubit[3] q;\ng q[0];\n", {}),
    ("call_same_qubit", V3 + "gate g a, b { cx a, b; }\nqubit[2] q;\ng q[1], q[1];\n", {}),
    ("physical_then_declared", V3 + "h $1;\nqubit q;\n", {}),
    ("while_loop", V3 + "qubit q;\nwhile (true) { x q; }\n", {}),
    ("opaque", V2 + "opaque g a;\n", {}),
]


def main(ref_src: str) -> None:
    sys.path.insert(0, ref_src)
    import lucivant_sim as ls
    from lucivant_sim import qasm

    out = []
    for name, src, params in VALID + INVALID:
        rec: dict[str, object] = {"name": name, "source": src, "params": params}
        try:
            c = qasm.parse(src, params)
            rec["circuit"] = {
                "digest": c.digest(),
                "num_qubits": c.num_qubits,
                "num_clbits": c.num_clbits,
                "qregs": [[r.name, r.offset, r.size] for r in c.qregs],
                "cregs": [[r.name, r.offset, r.size] for r in c.cregs],
                "inputs": dict(c.inputs),
                "kinds": [type(op).__name__ for op in c.operations],
                "is_dynamic": c.is_dynamic(),
                "final_measurements": [list(p) for p in c.final_measurements()],
                "count_ops": c.count_ops(),
                "format_bits": [c.format_bits(b) for b in (0, 1, 5, (1 << c.num_clbits) - 1)] if c.num_clbits else [],
            }
        except Exception as exc:  # noqa: BLE001 - the class, message and position are the record
            rec["error"] = {"class": type(exc).__name__, "message": str(exc), "line": getattr(exc, "line", None),
                            "column": getattr(exc, "column", None)}  # fmt: skip
        out.append(rec)
    (HERE / "qasm.json").write_text(json.dumps({"reference_version": ls.__version__, "programs": out}, indent=1))
    bad = [r["name"] for r in out if r["name"] in dict((n, 1) for n, _, _ in VALID) and "error" in r]
    print("wrote", HERE / "qasm.json", len(out), "programs; valid programs Orrery refused:", bad)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden_qasm.py /path/to/lucivant-sim/src")
    main(sys.argv[1])
