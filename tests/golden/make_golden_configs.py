"""Generate the benchmark-size golden fixtures by running Orrery (lucivant-sim 0.3.0) itself.

Run from the repository root, in a checkout where Orrery's sources are readable:

    python tests/golden/make_golden_configs.py /path/to/lucivant-sim/src [--jobs 8]

The path to Orrery's ``src`` directory is required. The cases are the benchmark workloads at the
sizes they are benchmarked at (each case runs in its own spawned process; the slowest, a
12-qubit density matrix with a 16-operator Kraus channel on every u3, takes about 16 minutes on
one core):

* ``cfg2_plain``: 12 qubits x 12 brickwork layers (seed 7) with Orrery's uniform noise
  (1e-3, 1e-2, readout 2e-2) plus thermal relaxation on u3 (the replacing reading): the 4096
  probabilities, the 23 <Z> observables from the density matrix's diagonal, and one <Z_0> through
  ``ls.expectation``.
* ``cfg2_inst{i}``: batched noise instances 0, 1, 128 and 255 of the benchmark's 256 (seed 7): the
  composed thermal + depolarising channel on u3 as a custom Kraus channel, depolarising on cx; the
  same outputs. The noise digest is stored so the tests can check they build the same model.
* ``cfg3_serial64``: 18 qubits x 16 rounds of mid-circuit measurement (seed 7), uniform noise
  (1e-3, 1e-2), 64 shots with seed 7 in Orrery's per-shot draw order: counts, every shot's bits
  and the generator's state after the last shot.
* ``cfg4_full``: 2048 qubits x 1000 Clifford layers (seed 11), depolarising 1e-3 on every gate,
  readout 0.01 / 0.03, 1000 shots with seed 11: the counts digest, the number of ones per
  classical bit, the noiseless tableau's digest and x0.
* ``clifford_maps``: the Pauli-conjugation table of every gate name Orrery knows, at Clifford
  parameter values, and a 6-qubit tableau after a circuit over all of them.

Writes ``tests/golden/configs.json`` and ``tests/golden/configs.npz``; the tests never need
Orrery at run time.
"""

from __future__ import annotations

import argparse
import hashlib
import json
import math
import multiprocessing as mp
import os
import sys
import time
from pathlib import Path

os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")  # before numpy: one thread per case process
os.environ.setdefault("OMP_NUM_THREADS", "1")

import numpy as np  # noqa: E402

sys.dont_write_bytecode = True
HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]

QUBITS2, LAYERS2, SEED2, INSTANCES2 = 12, 12, 7, 256
BATCH_MEMBERS = (0, 1, 128, 255)


def _setup(ref_src: str):
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    sys.dont_write_bytecode = True
    if str(ROOT) not in sys.path:
        sys.path.insert(0, str(ROOT))
    if ref_src not in sys.path:
        sys.path.insert(0, ref_src)
    import lucivant_sim as ls

    return ls


def _z_from_diagonal(diag: np.ndarray, n: int) -> list[float]:
    """<Z_i> (i = 0..n-1) then <Z_i Z_i+1> (i = 0..n-2), as Tr(P rho) over the real diagonal."""
    idx = np.arange(1 << n)
    out = []
    for i in range(n):
        out.append(float(np.sum(diag * (1 - 2 * ((idx >> i) & 1)))))
    for i in range(n - 1):
        out.append(float(np.sum(diag * (1 - 2 * (((idx >> i) ^ (idx >> (i + 1))) & 1)))))
    return out


def _orrery_instance_noise(ls, single: float, two: float, readout: float):
    """Orrery's model of one batched instance: thermal relaxation (120, 90, 0.05) after a
    depolarising error of average infidelity ``single``, one Kraus channel on u3; depolarising
    ``two`` on two-qubit gates; readout ``readout``."""
    th = ls.thermal_relaxation(120, 90, 0.05)
    dp = ls.from_gate_error(single, 1)
    kraus = tuple(t @ d for d in dp.kraus for t in th.kraus)
    channel = ls.Channel("thermal_relaxation+depolarizing", 1, kraus, (120, 90, 0.05, dp.params[0]))
    return ls.NoiseModel.uniform(two=two, readout=readout).add_gate_error(channel, gates="u3")


def case_cfg2(ref_src: str, which: str) -> tuple[str, dict, dict]:
    ls = _setup(ref_src)
    from lucivant_sim.engines import DensityMatrix  # noqa: F401  (Orrery's engine, run by ls.*)

    from lucivant_sim_gb300 import workloads as wl

    src = wl.brickwork(QUBITS2, LAYERS2, seed=SEED2, measure=False)
    t0 = time.perf_counter()
    if which == "plain":
        noise = ls.NoiseModel.uniform(single=1e-3, two=1e-2, readout=2e-2).add_gate_error(
            ls.thermal_relaxation(t1=120, t2=90, time=0.05), gates="u3"
        )
        info: dict = {}
    else:
        member = int(which)
        rng = np.random.default_rng(SEED2)
        singles = rng.uniform(1e-4, 5e-3, size=INSTANCES2)
        twos = rng.uniform(1e-3, 3e-2, size=INSTANCES2)
        noise = _orrery_instance_noise(ls, float(singles[member]), float(twos[member]), 2e-2)
        info = {"member": member, "instances": INSTANCES2, "noise_seed": SEED2,
                "single": float(singles[member]), "two": float(twos[member])}
    rho = ls.density_matrix(src, noise)
    seconds = time.perf_counter() - t0
    diag = np.real(np.diagonal(rho)).copy()
    probs = np.clip(diag, 0.0, None)
    name = f"cfg2_{which}" if which == "plain" else f"cfg2_inst{int(which)}"
    meta = dict(info, qasm_args=[QUBITS2, LAYERS2, SEED2], noise_digest=noise.digest(), z=_z_from_diagonal(diag, QUBITS2),
                orrery_seconds=seconds, trace=float(diag.sum()))  # fmt: skip
    return name, meta, {f"{name}_probs": probs}


def case_cfg2_expectation(ref_src: str) -> tuple[str, dict, dict]:
    ls = _setup(ref_src)
    from lucivant_sim_gb300 import workloads as wl

    src = wl.brickwork(QUBITS2, LAYERS2, seed=SEED2, measure=False)
    noise = ls.NoiseModel.uniform(single=1e-3, two=1e-2, readout=2e-2).add_gate_error(
        ls.thermal_relaxation(t1=120, t2=90, time=0.05), gates="u3"
    )
    label = "I" * (QUBITS2 - 1) + "Z"
    t0 = time.perf_counter()
    value = ls.expectation(src, label, noise)
    return "cfg2_plain_expectation", {"label": label, "value": float(value),
                                      "orrery_seconds": time.perf_counter() - t0}, {}  # fmt: skip


def case_cfg3(ref_src: str) -> tuple[str, dict, dict]:
    ls = _setup(ref_src)
    from lucivant_sim import simulator as osim

    from lucivant_sim_gb300 import workloads as wl

    src = wl.midcircuit(18, 16, seed=7)
    noise = ls.NoiseModel.uniform(single=1e-3, two=1e-2)
    shots, seed = 64, 7
    t0 = time.perf_counter()
    result = ls.run(src, shots=shots, seed=seed, noise=noise, method="trajectories")
    seconds = time.perf_counter() - t0
    circuit = ls.parse(src)
    rng = np.random.default_rng(seed)
    bits = [int(osim._trajectory(circuit, noise, rng)) for _ in range(shots)]
    state = rng.bit_generator.state["state"]
    meta = {"qasm_args": [18, 16, 7], "shots": shots, "seed": seed, "counts": result.counts,
            "method": result.method, "counts_digest": result.counts_digest, "noise_digest": noise.digest(),
            "shot_bits": bits, "rng_state": str(state["state"]), "rng_inc": str(state["inc"]),
            "orrery_seconds": seconds}  # fmt: skip
    return "cfg3_serial64", meta, {}


def case_cfg4(ref_src: str) -> tuple[str, dict, dict]:
    ls = _setup(ref_src)
    from lucivant_sim import stabilizer as stab

    from lucivant_sim_gb300 import workloads as wl

    n, layers, shots, seed = 2048, 1000, 1000, 11
    src = wl.clifford_layers(n, layers, seed=seed)
    noise = ls.NoiseModel()
    noise.add_gate_error(ls.depolarizing(1e-3, 1)).add_gate_error(ls.depolarizing(1e-3, 2))
    noise.add_readout_error(ls.ReadoutError(0.01, 0.03))
    t0 = time.perf_counter()
    circuit = ls.parse(src)
    parse_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    result = ls.run(circuit, shots=shots, seed=seed, noise=noise)
    run_s = time.perf_counter() - t0
    ones = np.zeros(n, dtype=np.int64)
    for key, count in result.counts.items():  # key: clbit n-1 first
        ones += count * (np.frombuffer(key.encode(), dtype=np.uint8)[::-1] == ord("1"))
    from lucivant_sim.circuit import Gate

    tab = stab.Tableau(n)
    for op in circuit.operations:
        if isinstance(op, Gate):
            tab.apply(stab.clifford_map(op.matrix), op.qubits)
    digest = hashlib.sha256(tab.x.tobytes() + tab.z.tobytes() + tab.r.tobytes()).hexdigest()
    x0, basis = tab.copy().support(list(range(n)))
    meta = {"qasm_args": [n, layers, seed], "shots": shots, "seed": seed, "method": result.method,
            "counts_digest": result.counts_digest, "distinct": len(result.counts), "noise_digest": noise.digest(),
            "circuit_digest": result.circuit_digest, "tableau_sha256": digest, "basis_rows": int(len(basis)),
            "basis_sha256": hashlib.sha256(np.ascontiguousarray(basis, dtype=np.uint8).tobytes()).hexdigest(),
            "orrery_parse_seconds": parse_s, "orrery_run_seconds": run_s}  # fmt: skip
    return "cfg4_full", meta, {"cfg4_ones": ones, "cfg4_x0": np.asarray(x0, dtype=np.uint8)}


def _clifford_params(nparams: int) -> list[tuple[float, ...]]:
    """Parameter tuples at which a parametrised gate is Clifford (multiples of pi/2)."""
    if nparams == 0:
        return [()]
    choices = [math.pi / 2, math.pi, -math.pi / 2, 0.0]
    out = []
    for i in range(3):
        out.append(tuple(choices[(i + j) % len(choices)] for j in range(nparams)))
    return out


def case_clifford(ref_src: str) -> tuple[str, dict, dict]:
    ls = _setup(ref_src)
    from lucivant_sim import stabilizer as stab
    from lucivant_sim.gates import GATES

    maps: dict = {}
    arrays: dict = {}
    program: list = []
    rng = np.random.default_rng(3)
    for name in sorted(GATES):
        spec = GATES[name]
        for params in _clifford_params(spec.params):
            m = spec.matrix(*params)
            cmap = stab.clifford_map(np.asarray(m, dtype=np.complex128))
            if cmap is None:
                continue
            key = f"{name}({','.join(repr(p) for p in params)})"
            maps[key] = {"name": name, "params": list(params), "k": int(cmap.k), "kind": stab._kind(cmap)}
            arrays[f"cmap_bits::{key}"] = cmap.bits
            arrays[f"cmap_sign::{key}"] = cmap.sign
            qs = [int(q) for q in rng.permutation(6)[: spec.qubits]]
            program.append((key, name, list(params), qs))
    # one circuit over every Clifford gate, twice in a shuffled order, on 6 qubits from |0..0>
    order = list(range(len(program))) + [int(i) for i in rng.permutation(len(program))]
    tab = stab.Tableau(6)
    applied = []
    for i in order:
        key, name, params, qs = program[i]
        m = np.asarray(GATES[name].matrix(*params), dtype=np.complex128)
        tab.apply(stab.clifford_map(m), tuple(qs))
        applied.append([name, params, qs])
    arrays["cliff6_x"], arrays["cliff6_z"], arrays["cliff6_r"] = tab.x.copy(), tab.z.copy(), tab.r.copy()
    return "clifford_maps", {"maps": maps, "program": applied}, arrays


def _run(task: tuple) -> tuple[str, dict, dict, float]:
    fn, args = task
    t0 = time.perf_counter()
    name, meta, arrays = globals()[fn](*args)
    return name, meta, arrays, time.perf_counter() - t0


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("orrery_src", help="path to Orrery's src directory (the one holding lucivant_sim/)")
    ap.add_argument("--jobs", type=int, default=8)
    ap.add_argument("--only", default="", help="comma-separated case names (default: all)")
    args = ap.parse_args()
    src = str(Path(args.orrery_src).resolve())
    tasks = [("case_cfg2", (src, str(m))) for m in BATCH_MEMBERS]
    tasks += [("case_cfg2", (src, "plain")), ("case_cfg2_expectation", (src,)), ("case_cfg4", (src,)),
              ("case_cfg3", (src,)), ("case_clifford", (src,))]  # fmt: skip
    if args.only:
        keep = set(args.only.split(","))
        tasks = [t for t in tasks if t[0] in keep or (t[0] == "case_cfg2" and f"cfg2_{t[1][1]}" in keep)]
    out_json, out_npz = HERE / "configs.json", HERE / "configs.npz"
    meta: dict = {"cases": {}}
    arrays: dict = {}
    if out_json.exists() and args.only:  # merge into the existing fixtures
        meta = json.loads(out_json.read_text())
        with np.load(out_npz) as data:
            arrays = {k: data[k] for k in data.files}
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(args.jobs, len(tasks))) as pool:
        for name, m, a, seconds in pool.imap_unordered(_run, tasks):
            print(f"{name}: {seconds:.0f} s", flush=True)
            meta["cases"][name] = m
            arrays.update(a)
    _setup(src)
    import lucivant_sim as ls

    meta["reference_version"] = ls.__version__
    np.savez_compressed(out_npz, **arrays)
    out_json.write_text(json.dumps(meta, indent=1, sort_keys=True))
    print("wrote", out_npz, out_json)


if __name__ == "__main__":
    main()
