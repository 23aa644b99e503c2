"""Record parts of Orrery's public surface (lucivant-sim 0.3.0) that need no simulation, by running
Orrery itself: every gate's matrix at seeded parameters and its canonical name, the ``Result``
record (fingerprint, counts digest, dictionary form, frequencies, most frequent outcome) of
synthetic results, and the command line's help, version and argument errors.

Run from the repository root, in a checkout where Orrery's sources are readable:

    python tests/golden/make_golden_api.py /path/to/lucivant-sim/src

It writes ``tests/golden/api.json`` and ``tests/golden/api.npz``. The tests never need Orrery.
"""

from __future__ import annotations

import contextlib
import io
import json
import os
import sys
from pathlib import Path

import numpy as np

sys.dont_write_bytecode = True
HERE = Path(__file__).resolve().parent
COLUMNS = "100"  # argparse wraps help text to the terminal width

RESULTS = [
    {"counts": {"00": 480, "11": 520}, "shots": 1000, "seed": 7, "method": "statevector", "num_qubits": 2,
     "num_clbits": 2, "circuit_digest": "sha256:" + "ab" * 32, "noise_digest": None, "version": "0.3.0",
     "elapsed_seconds": 0.012345},
    {"counts": {"0 10": 3, "1 01": 5, "1 10": 5}, "shots": 13, "seed": 0, "method": "trajectories",
     "num_qubits": 3, "num_clbits": 3, "circuit_digest": "sha256:" + "01" * 32,
     "noise_digest": "sha256:" + "fe" * 32, "version": "0.3.0", "elapsed_seconds": 1.5},
    {"counts": {}, "shots": 0, "seed": 2**62, "method": "stabilizer", "num_qubits": 2048, "num_clbits": 0,
     "circuit_digest": "sha256:" + "00" * 32, "noise_digest": None, "version": "0.3.0+gb300-1",
     "elapsed_seconds": 0.0},
]  # fmt: skip

CLI_ARGS = [
    ["--help"], ["--version"], ["run", "--help"], ["state", "--help"], ["expect", "--help"], ["verify", "--help"],
    [], ["run"], ["run", "x.qasm", "--shots", "many"], ["run", "x.qasm", "--method", "fast"], ["bogus"],
    ["expect", "x.qasm"],
]  # fmt: skip


def _cli(main, argv: list[str]) -> dict:
    out, err = io.StringIO(), io.StringIO()
    code = None
    with contextlib.redirect_stdout(out), contextlib.redirect_stderr(err):
        try:
            code = main(argv)
        except SystemExit as exc:
            code = exc.code
    return {"argv": argv, "code": code, "stdout": out.getvalue(), "stderr": err.getvalue()}


def main(ref_src: str) -> None:
    os.environ["COLUMNS"] = COLUMNS
    sys.path.insert(0, ref_src)
    import lucivant_sim as ls
    from lucivant_sim import cli, gates
    from lucivant_sim.simulator import Result

    arrays: dict[str, np.ndarray] = {}
    rng = np.random.default_rng(17)
    names = sorted(gates.GATES)
    gate_rec = []
    for name in names:
        spec = gates.GATES[name]
        params = [float(v) for v in rng.uniform(-7, 7, size=spec.params)]
        arrays[f"gate::{name}"] = np.asarray(gates.gate_matrix(name, tuple(params)), dtype=np.complex128)
        gate_rec.append({"name": name, "params": params, "qubits": spec.qubits, "canonical": gates.canonical_name(name)})
    powers = []
    for i, (name, k) in enumerate([("sx", 0.5), ("h", 2.0), ("t", -1.5), ("rx", 0.3), ("s", 3)]):
        u = gates.gate_matrix(name, tuple([0.7] * gates.GATES[name].params))
        arrays[f"power::{i}"] = np.asarray(gates.matrix_power(u, k), dtype=np.complex128)
        powers.append({"name": name, "k": k})
    results = []
    for fields in RESULTS:
        r = Result(**fields)
        results.append({"fields": fields, "fingerprint": r.fingerprint, "counts_digest": r.counts_digest,
                        "to_dict": r.to_dict(), "frequencies": r.frequencies(), "most_frequent": r.most_frequent()})  # fmt: skip
    clis = [_cli(cli.main, argv) for argv in CLI_ARGS]
    out = {"reference_version": ls.__version__, "columns": COLUMNS, "gates": gate_rec, "powers": powers,
           "results": results, "cli": clis}  # fmt: skip
    np.savez_compressed(HERE / "api.npz", **arrays)
    (HERE / "api.json").write_text(json.dumps(out, indent=1, sort_keys=True))
    print("wrote", HERE / "api.json", HERE / "api.npz")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden_api.py /path/to/lucivant-sim/src")
    main(sys.argv[1])
