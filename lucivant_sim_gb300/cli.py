"""Command-line front end on the GB300 engine, with Orrery's commands, options, output and exit
codes (``src/lucivant_sim/cli.py:1-128``):

    python -m lucivant_sim_gb300 run bell.qasm --shots 2000 --seed 7
    python -m lucivant_sim_gb300 run bell.qasm --noise device.json --json > result.json
    python -m lucivant_sim_gb300 verify result.json bell.qasm --noise device.json
    python -m lucivant_sim_gb300 state bell.qasm --amplitudes
    python -m lucivant_sim_gb300 expect bell.qasm ZZ

Exit status: 0 on success, 1 when ``verify`` finds a mismatch, 2 on a program, noise, argument or
engine error (one line ``lucivant-sim: <message>`` on standard error).
"""

from __future__ import annotations

import argparse
import json
import sys
from collections.abc import Callable, Sequence
from pathlib import Path
from typing import Any

from lucivant_sim_gb300._lib import EngineError, SimulationError
from lucivant_sim_gb300.noise import NoiseModel
from lucivant_sim_gb300.qasm import QasmError, load, parse
from lucivant_sim_gb300.simulator import METHODS, __version__, expectation, probabilities, run, statevector, verify

PROG = "lucivant-sim"
BAR_WIDTH = 32
STATE_ROWS = 64  # most probable outcomes `state` lists
AMPLITUDE_FLOOR = 1e-12  # amplitudes `state --amplitudes` leaves out


def bar(p: float) -> str:
    """A horizontal bar of ``round(p * 32)`` full blocks."""
    return "█" * round(p * BAR_WIDTH)


def parse_params(items: Sequence[str]) -> dict[str, float]:
    """``--param NAME=VALUE`` items as a mapping (a malformed item ends the program)."""
    params: dict[str, float] = {}
    for item in items:
        name, eq, value = item.partition("=")
        if not eq:
            raise SystemExit(f"--param needs name=value, not {item!r}")
        params[name.strip()] = float(value)
    return params


def read_program(source: str, params: dict[str, float]) -> Any:
    """The circuit in file ``source``, or on standard input for ``-``."""
    return parse(sys.stdin.read(), params) if source == "-" else load(Path(source), params)


def noise_of(args: argparse.Namespace) -> NoiseModel | None:
    """A calibration file wins over the uniform error rates; no noise when neither is given."""
    if getattr(args, "noise", None):
        return NoiseModel.from_calibration(args.noise)
    rates = (getattr(args, "single", 0.0), getattr(args, "two", 0.0), getattr(args, "readout", 0.0))
    return NoiseModel.uniform(*rates) if any(rates) else None


def _add_program(p: argparse.ArgumentParser) -> None:
    p.add_argument("program", help="an OpenQASM 2 or 3 file, or - for standard input")
    p.add_argument("--param", action="append", default=[], metavar="NAME=VALUE", help="an input parameter")
    p.add_argument("--noise", metavar="FILE", help="a device calibration (Lucivant twin JSON)")
    p.add_argument("--single", type=float, default=0.0, help="uniform one-qubit gate error")
    p.add_argument("--two", type=float, default=0.0, help="uniform two-qubit gate error")
    p.add_argument("--readout", type=float, default=0.0, help="uniform readout error")


def build_parser() -> argparse.ArgumentParser:
    parser = argparse.ArgumentParser(prog=PROG, description="Lucivant Orrery: a quantum circuit simulator.")
    parser.add_argument("--version", action="version", version=f"{PROG} {__version__}")
    commands = parser.add_subparsers(dest="command", required=True)

    p = commands.add_parser("run", help="sample measurement counts")
    _add_program(p)
    p.add_argument("--shots", type=int, default=1024)
    p.add_argument("--seed", type=int)
    p.add_argument("--method", choices=METHODS, default="automatic")
    p.add_argument("--json", action="store_true", help="print the full result as JSON")

    p = commands.add_parser("state", help="exact probabilities (and amplitudes for ideal circuits)")
    _add_program(p)
    p.add_argument("--amplitudes", action="store_true")

    p = commands.add_parser("expect", help="exact expectation of a Pauli observable")
    _add_program(p)
    p.add_argument("observable", help='a Pauli string such as ZZ, or JSON like {"ZI": 0.5, "XX": 1}')

    p = commands.add_parser("verify", help="rerun a saved --json result and check it matches")
    p.add_argument("result", help="the saved result JSON")
    _add_program(p)
    return parser


def cmd_run(args: argparse.Namespace, program: Any, noise: NoiseModel | None, out: Callable[[str], None]) -> int:
    result = run(program, args.shots, seed=args.seed, noise=noise, method=args.method)
    if args.json:
        out(json.dumps(result.to_dict(), indent=2))
        return 0
    out(f"{result.num_qubits} qubits · {result.shots} shots · {result.method} · seed {result.seed}")
    # most frequent first, ties by outcome string
    for key, count in sorted(result.counts.items(), key=lambda kv: (-kv[1], kv[0])):
        out(f"  {key or '(no bits)'}  {count:>8}  {bar(count / max(result.shots, 1))}")
    if not result.counts:
        out("  The program measures nothing; try `lucivant-sim state`.")
    out(f"fingerprint {result.fingerprint}")
    return 0


def cmd_state(args: argparse.Namespace, program: Any, noise: NoiseModel | None, out: Callable[[str], None]) -> int:
    probs = probabilities(program, noise)
    for key, p in sorted(probs.items(), key=lambda kv: -kv[1])[:STATE_ROWS]:
        out(f"  {key}  {p:.6f}  {bar(p)}")
    if args.amplitudes:
        if noise is not None and noise.has_gate_errors():
            raise SimulationError("amplitudes exist only for ideal circuits")
        vec = statevector(program)
        width = max(1, (len(vec) - 1).bit_length())
        for index, amp in enumerate(vec):
            if abs(amp) > AMPLITUDE_FLOOR:
                out(f"  |{index:0{width}b}>  {amp.real:+.6f}{amp.imag:+.6f}i")
    return 0


def cmd_expect(args: argparse.Namespace, program: Any, noise: NoiseModel | None, out: Callable[[str], None]) -> int:
    text = args.observable.strip()
    observable = json.loads(text) if text.startswith("{") else text
    out(f"{expectation(program, observable, noise):.10g}")
    return 0


def cmd_verify(args: argparse.Namespace, program: Any, noise: NoiseModel | None, out: Callable[[str], None]) -> int:
    if verify(args.result, program, noise):
        out("verified: the rerun matches the saved counts")
        return 0
    out("MISMATCH: the rerun differs")
    return 1


COMMANDS: dict[str, Callable[..., int]] = {"run": cmd_run, "state": cmd_state, "expect": cmd_expect, "verify": cmd_verify}


def main(argv: Sequence[str] | None = None) -> int:
    args = build_parser().parse_args(argv)
    try:
        program = read_program(args.program, parse_params(args.param))
        return COMMANDS[args.command](args, program, noise_of(args), print)
    except (QasmError, SimulationError, EngineError, ValueError, OSError, TypeError) as exc:
        print(f"{PROG}: {exc}", file=sys.stderr)
        return 2


if __name__ == "__main__":  # pragma: no cover
    raise SystemExit(main())
