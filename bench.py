#!/usr/bin/env python3
"""Benchmark: the batched noisy density-matrix hot path on one GB300 (per rank).

Workload (one step): 256 noise instances of a 12-qubit, 12-layer u3+cx brickwork circuit (angles
U[0, 2π) from seed 7), each with thermal relaxation (T1 = 120, T2 = 90, t = 0.05) composed with a
depolarising one-qubit error ~ U[1e-4, 5e-3] on every u3, depolarising two-qubit error
~ U[1e-3, 3e-2] on every cx, evolved as one 256-member register of density matrices in the
Pauli-transfer form from |0><0| through passes compiled for the circuit at run time, then the
exact probabilities and the 23 observables <Z_i>, <Z_i Z_i+1> of every instance. The default
precision is the reference's: complex128 requests run the Pauli-transfer register in real64
(FP64 arithmetic, 32 GiB); ``--precision c64`` runs it in real32 (16 GiB). Both registers are
larger than L2 (no flush needed).

metric: circuits/s — density-matrix instances evolved and reduced per second, whole job. Beside
it: the HBM bytes the passes move per second, the roofline of the passes (FP64 arithmetic for
the real64 register, which bounds it on this GPU; HBM for real32), the results of instances 0,
1, 128 and 255 against Orrery's own (committed fixtures, made by running Orrery), the end-to-end
rate through the public batched call (host inputs, host results), the complex64 batched run with
its error, and the plain single-instance complex128 path on the same GPU.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun each rank runs its own 256 instances on its own GPU (weak scaling, no data-path
collective). ``--impl reference`` times the CPU port of Orrery's algorithm (the oracle) on the
host cores instead, on rank 0 only, without loading the engine library.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

QUBITS, LAYERS, SEED, INSTANCES = 12, 12, 7, 256
FALLBACK_HBM_GBS = 6800.0
GOLDEN_MEMBERS = (0, 1, 128, 255)  # instances with Orrery-made fixtures (tests/golden/configs.*)
CPU_SAMPLE_U3, CPU_SAMPLE_CX = 3, 2  # whole gate+channel operations timed for the CPU baseline
REF_BUDGET_S = 120.0  # timed seconds of the reference arm, spread over its steps


def parse_args() -> argparse.Namespace:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--precision", choices=("c128", "c64", "df64"), default="c128",
                    help="c128: real64 Pauli-transfer register (FP64); c64: real32; df64: double-float pairs")
    ap.add_argument("--instances", type=int, default=INSTANCES)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-c64", action="store_true", help="skip the complex64 batched run beside the headline")
    ap.add_argument("--no-autotune", action="store_true", help="default plan choices (no autotuner search)")
    ap.add_argument("--ref-full", type=int, default=0, metavar="N",
                    help="reference arm: evolve N whole instances (one per host process) instead of timed samples")
    ap.add_argument("--workload", choices=("dm-batch", "serve", "sv20", "traj18", "stab2048"), default="dm-batch",
                    help="dm-batch: the batched density-matrix step (default); serve: the served mix; sv20: "
                    "statevector 20q x 20 layers; traj18: trajectories 18q x 16 rounds x 4096 shots; stab2048: "
                    "stabilizer 2048q x 1000 layers x 1000 shots")  # fmt: skip
    ap.add_argument("--jobs", type=int, default=400, help="serve: jobs in the served mix")
    ap.add_argument("--rate", type=float, default=200.0, help="serve: offered arrivals per second")
    ap.add_argument("--serve-workers", type=int, default=16, help="serve: device worker slots")
    return ap.parse_args()


def _plain(o):
    """numpy scalars and arrays in a bench line as plain JSON values."""
    import numpy as np

    if isinstance(o, np.generic):
        return o.item()
    if isinstance(o, np.ndarray):
        return o.tolist()
    raise TypeError(f"Object of type {type(o).__name__} is not JSON serializable")


def dist_info() -> tuple[int, int, int]:
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Dist:
    """Barrier and max-over-ranks on the host (gloo) when launched by torchrun. A rank that never
    joins, or leaves, ends the others' next collective with an error after ``timeout_s``."""

    def __init__(self, world: int, timeout_s: float = 600.0) -> None:
        self.world = world
        if world > 1:
            import datetime

            import torch.distributed as td

            td.init_process_group("gloo", timeout=datetime.timedelta(seconds=timeout_s))
            self.td = td

    def barrier(self) -> None:
        if self.world > 1:
            self.td.barrier()

    def max(self, value: float) -> float:
        if self.world == 1:
            return value
        import torch

        t = torch.tensor([value], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self) -> None:
        if self.world > 1:
            self.td.destroy_process_group()


class Clocks:
    """nvidia-smi samples every 200 ms while running (SM clock, throttle reasons)."""

    QUERY = (
        "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
        "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
        "clocks_event_reasons.sw_power_cap,utilization.gpu"
    )

    def __init__(self, gpu: int) -> None:
        self.gpu = gpu
        self.proc: subprocess.Popen | None = None

    def start(self) -> None:
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)  # fmt: skip
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, util, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9], strict=True):
                if val.lower().startswith("active"):
                    reasons.add(name)
            if len(f) > 9:
                try:
                    util.append(float(f[9]))
                except ValueError:
                    pass
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
            "gpu_util_median_pct": statistics.median(util) if util else None,
        }


def measured_peak() -> tuple[float, str]:
    path = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(path.read_text())["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(tag: str) -> list[float] | None:
    """DRAM bytes (read + write) per pass of a full-size launch, from the committed ncu summary
    (an 8-instance capture scaled by the members), or None."""
    path = ROOT / "profiles" / f"tile_pass_dm12_{tag}.md"
    if not path.exists():
        return None
    for line in path.read_text().splitlines():
        if line.startswith("traffic_bytes_per_pass:"):
            return [float(x) for x in line.split(":", 1)[1].split(",")]
    return None


def fp64_peak_tflops() -> float:
    """FP64 rate of cuBLAS (torch float64 matmul, 4096^3, best of 5) on this GPU: the measured
    denominator of the real64 passes' arithmetic roofline."""
    import torch

    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    best = float("inf")
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1000.0)
    del a, b
    torch.cuda.empty_cache()
    return 2.0 * n**3 / best / 1e12


def workload():
    """The circuit (pure host code: no engine library) and the 23 Z observables."""
    from lucivant_sim_gb300 import qasm, workloads as wl

    circuit = qasm.parse(wl.brickwork(QUBITS, LAYERS, seed=SEED, measure=False))
    return circuit, wl.z_observables(QUBITS)


def load_golden() -> dict:
    """Orrery's results for instances 0, 1, 128 and 255 of the benchmark (committed fixtures made
    by running Orrery itself); empty when absent."""
    import numpy as np

    meta_path, arr_path = ROOT / "tests" / "golden" / "configs.json", ROOT / "tests" / "golden" / "configs.npz"
    if not (meta_path.exists() and arr_path.exists()):
        return {}
    cases = json.loads(meta_path.read_text())["cases"]
    out = {}
    with np.load(arr_path) as data:
        for m in GOLDEN_MEMBERS:
            name = f"cfg2_inst{m}"
            if name in cases and f"{name}_probs" in data.files:
                out[m] = {"probs": data[f"{name}_probs"], "z": np.asarray(cases[name]["z"]),
                          "noise_digest": cases[name].get("noise_digest")}
    return out


def golden_errors(probs, exps, golden: dict, noises: list) -> dict:
    """Max-abs probability and <Z> errors and probability TVD against Orrery, per fixture member
    whose noise model is the one Orrery ran (same digest): another instance count draws other
    noise parameters, and those members are listed as not comparable."""
    import numpy as np

    per, other = {}, []
    for m, g in golden.items():
        if m >= probs.shape[0]:
            continue
        if g.get("noise_digest") != noises[m].digest():
            other.append(m)
            continue
        per[str(m)] = {
            "max_abs_probability": float(np.max(np.abs(probs[m] - g["probs"]))),
            "probability_tvd": 0.5 * float(np.abs(probs[m] - g["probs"]).sum()),
            "max_abs_z": float(np.max(np.abs(exps[:, m] - g["z"]))),
        }
    worst = {k: max(v[k] for v in per.values()) for k in ("max_abs_probability", "probability_tvd", "max_abs_z")} if per else {}
    out = {"members": per, "worst": worst, "against": "Orrery 0.3.0 run on the same instances (tests/golden/configs.*)"}
    if other:
        out["not_comparable"] = {"members": other, "why": "other noise parameters than Orrery's run (the instance "
                                 "count changes the seeded draws)"}
    return out


# ------------------------------------------------------------------------------ CPU legs


def _oracle_ops(args: tuple[int, int, int]) -> tuple[float, int, int]:
    """Evolve operations [start, start + count) (gate then its channel, circuit order, wrapping
    around) of instance ``instance`` with the oracle on a full-size 12-qubit density matrix from
    |0><0|; returns (seconds, operations done, operations per circuit). Host code only: the engine
    library is never loaded here."""
    instance, start, count = args
    import numpy as np

    from lucivant_sim_gb300 import workloads as wl
    from oracle import dense

    circuit, _ = workload()
    noise = wl.dm_noise_instances(INSTANCES, seed=SEED)[instance % INSTANCES]
    n = QUBITS
    gates = [op for op in circuit.operations if op.kind == "gate"]
    rho = np.zeros(1 << (2 * n), dtype=np.complex128)
    rho[0] = 1
    t0 = time.perf_counter()
    for j in range(count):
        op = gates[(start + j) % len(gates)]
        rho = dense.apply_bits(rho, 2 * n, op.matrix, [n + q for q in op.qubits])
        rho = dense.apply_bits(rho, 2 * n, op.matrix.conj(), list(op.qubits))
        ch = noise.gate_error(op.name, op.qubits)
        if ch is not None:
            rho = dense.dm_channel(rho, n, ch, op.qubits)
    return time.perf_counter() - t0, count, len(gates)


def _oracle_instance(instance: int) -> tuple[float, float]:
    """One whole instance with the oracle (gate, channel, then the probabilities); returns
    (seconds, probability of |0...0>)."""
    from lucivant_sim_gb300 import workloads as wl
    from oracle import dense

    circuit, _ = workload()
    noise = wl.dm_noise_instances(INSTANCES, seed=SEED)[instance % INSTANCES]
    t0 = time.perf_counter()
    probs = dense.probabilities_array(circuit, noise)
    return time.perf_counter() - t0, float(probs[0])


def _mapped_libraries() -> list[str]:
    """This repository's shared objects mapped into the process (Linux /proc/self/maps)."""
    try:
        text = Path("/proc/self/maps").read_text()
    except OSError:
        return []
    return sorted({line.split()[-1] for line in text.splitlines() if line.endswith(".so") and str(ROOT) in line})


def cpu_baseline() -> dict:
    """The oracle (a port of Orrery's algorithm) on one host thread, on a bounded sample: the
    first u3 and cx gate+channel operations of instance 0, projected to the whole circuit."""
    code = (
        "import sys, json; sys.path.insert(0, %r); import bench; "
        "a = bench._oracle_ops((0, 0, %d)); b = bench._oracle_ops((0, 12, %d)); "
        "print(json.dumps([a, b]))" % (str(ROOT), CPU_SAMPLE_U3, CPU_SAMPLE_CX)
    )
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1")
    t0 = time.perf_counter()
    proc = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=900)
    wall = time.perf_counter() - t0
    if proc.returncode != 0:
        return {"value": None, "unit": "circuits/s", "error": proc.stderr.strip()[-300:]}
    (s1, k1, total), (s2, k2, _) = json.loads(proc.stdout.strip().splitlines()[-1])
    circuit, _ = workload()
    gates = [op for op in circuit.operations if op.kind == "gate"]
    n1 = sum(1 for g in gates if len(g.qubits) == 1)
    per_circuit = n1 * s1 / k1 + (len(gates) - n1) * s2 / k2
    return {
        "value": 1.0 / per_circuit,
        "unit": "circuits/s",
        "cores": 1,
        "kind": "port",
        "sample": f"oracle (port of Orrery's density-matrix algorithm), instance 0 at full size: {k1} u3 and {k2} cx "
        f"gate+channel operations timed whole ({wall:.1f} s wall), projected to the circuit's {n1} u3 and "
        f"{len(gates) - n1} cx: {per_circuit:.0f} s per instance",
    }


def reference_arm(args: argparse.Namespace) -> None:
    """The oracle port of Orrery's algorithm on every host core (one process per core, one thread
    each), on the benchmark's workload. Each step, every process evolves whole gate+channel
    operations of its own instance at full size; circuits counted = operations done / operations
    per circuit (a projection from measured whole operations, labelled so). ``--ref-full N``
    evolves N whole instances instead (no projection). The engine library is not loaded."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    import multiprocessing as mp

    cores = os.cpu_count() or 1
    os.environ["OPENBLAS_NUM_THREADS"] = "1"  # inherited by the spawned workers: one thread each
    os.environ["OMP_NUM_THREADS"] = "1"
    ctx = mp.get_context("spawn")
    base = {
        "impl": "reference",
        "metric": "circuits/s",
        "unit": "circuits/s",
        "n_gpus": args.gpus,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "c128",
        "data": "synthetic",
        "config": config_block(args),
    }
    if args.ref_full:
        procs = min(cores, args.ref_full)
        with ctx.Pool(procs) as pool:
            t0 = time.perf_counter()
            res = pool.map(_oracle_instance, range(args.ref_full))
            wall = time.perf_counter() - t0
        value = args.ref_full / wall
        line = dict(base, value=value, steps=1, warmup=0, ms_per_step=1000 * wall,
                    instance_seconds=[r[0] for r in res],
                    cpu_baseline={"value": value, "unit": "circuits/s", "cores": procs, "kind": "port",
                                  "sample": f"{args.ref_full} whole instances on {procs} processes (no projection)"},
                    e2e={"value": value, "unit": "circuits/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                    native_so_loaded=_mapped_libraries())  # fmt: skip
        print(json.dumps(line, default=_plain), flush=True)
        return
    with ctx.Pool(cores) as pool:
        warm = []
        for w in range(max(args.warmup, 1)):  # one whole operation per process (the first u3, first cx)
            warm += pool.map(_oracle_ops, [(i, 12 * (w % 2), 1) for i in range(cores)])
        t_op = statistics.mean(s / max(k, 1) for s, k, _ in warm)
        per_step = max(1, round(REF_BUDGET_S / max(args.steps, 1) / t_op))
        step_s, circuits, cursor = [], 0.0, 0
        for _ in range(args.steps):
            t0 = time.perf_counter()
            res = pool.map(_oracle_ops, [(i, cursor, per_step) for i in range(cores)])
            step_s.append(time.perf_counter() - t0)
            circuits += sum(k / total for _, k, total in res)
            cursor += per_step
    elapsed = sum(step_s)
    value = circuits / elapsed
    line = dict(base, value=value, steps=args.steps, warmup=args.warmup, ms_per_step=1000 * elapsed / args.steps,
                cpu_baseline={"value": value, "unit": "circuits/s", "cores": cores, "kind": "port",
                              "sample": f"each step: {cores} processes (one thread each), each evolving {per_step} whole "
                              "gate+channel operations of its own instance on a full-size 12-qubit density matrix with "
                              "the oracle; circuits = operations done / 210 per circuit (a projection from measured "
                              "whole operations)"},
                e2e={"value": value, "unit": "circuits/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                native_so_loaded=_mapped_libraries())  # fmt: skip
    print(json.dumps(line, default=_plain), flush=True)


def config_block(args: argparse.Namespace) -> dict:
    elem = 4 if args.precision == "c64" else 8
    return {
        "workload": f"density_matrix {QUBITS}q x {LAYERS} brickwork layers, {args.instances} noise instances per GPU",
        "qubits": QUBITS,
        "layers": LAYERS,
        "instances_per_gpu": args.instances,
        "precision": args.precision,
        "noise": "thermal_relaxation(120, 90, 0.05) composed with depolarising U[1e-4,5e-3] on u3; "
        "depolarising U[1e-3,3e-2] on cx; readout 2e-2",
        "outputs": "probabilities (2^12) and 23 Z observables per instance",
        # the workload's gates act on at most two qubits: the Pauli-transfer form, real64 for a
        # complex128 request (real32 for complex64)
        "form": "ptm",
        "l2": f"register {(elem * args.instances << 24) / 2**30:.0f} GiB > L2: no flush",
        "parallelism": f"replicas x{args.gpus} (independent instances per GPU)",
    }


# ------------------------------------------------------------------------------ GPU arm


def e2e_upload_bytes(circuit, noises) -> int:
    """Host-to-device bytes of one run_density_batch call: the operator table and data pool of
    each batch it evolves (two halves for an even batch)."""
    from lucivant_sim_gb300 import _lib, engine
    from lucivant_sim_gb300.batch import halves

    total = 0
    for part in halves(noises):
        ops = engine.ptm_oplist(circuit, part) if engine.dm_form(circuit, part) == "ptm" else engine.dm_oplist(circuit, part)
        total += ops.size * 16 + len(ops) * _lib.OP_DTYPE.itemsize
    return total


def timed_batch(batch, labels, steps: int, warmup: int, stream, local: int, dist) -> dict:
    """Warm-up, then ``steps`` timed steps (evolve + expectations + probabilities) bracketed by a
    barrier and device synchronisation, CUDA events on the register's stream, clocks sampled."""
    import numpy as np
    import torch

    def step(timed: list | None = None) -> tuple:
        if timed is None:
            batch.evolve()
        else:
            timed.append(batch.evolve_timed())
        return batch.expectations(labels), batch.probabilities()

    for _ in range(warmup):
        step()
    batch.reg.sync()
    dist.barrier()
    clocks = Clocks(local)
    clocks.start()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    pass_ms: list = []
    torch.cuda.synchronize()
    t_start.record(stream)
    for _ in range(steps):
        exps, probs = step(pass_ms)
    t_end.record(stream)
    t_end.synchronize()
    batch.reg.sync()
    clock_info = clocks.stop()
    dist.barrier()
    elapsed = dist.max(t_start.elapsed_time(t_end) / 1000.0)
    return {"elapsed": elapsed, "pass_ms": np.stack(pass_ms), "exps": exps, "probs": probs, "clocks": clock_info}


def pass_rooflines(batch, pass_ms, real64: bool, fp64_peak: float | None) -> dict:
    """Per pass and over the evolution: bytes moved and HBM rate (each pass against its own
    bytes), FP arithmetic rate; the binding roofline of the dominant kernel."""
    import numpy as np

    info = batch.program.pass_info()
    med = np.median(pass_ms.astype(np.float64), axis=0)  # ms per pass, median over the timed steps
    elem_bytes = batch.register_bytes // (batch.batch << (2 * batch.n))
    visited = info["bytes"] // (2 * elem_bytes)  # elements in the tiles each pass visits
    per_pass = []
    for i, ms in enumerate(med.astype(np.float64).tolist()):
        gbs = float(info["bytes"][i]) / (ms / 1000) / 1e9
        tflops = float(info["flops_per_element"][i]) * float(visited[i]) / (ms / 1000) / 1e12
        per_pass.append({"pass": i, "ms": round(float(ms), 4), "blocks": int(info["blocks"][i]),
                         "bytes": int(info["bytes"][i]), "hbm_gbs": round(gbs, 1),
                         "flops_per_element": float(info["flops_per_element"][i]), "tflops": round(tflops, 4)})  # fmt: skip
    total_s = float(med.sum()) / 1000
    moved = float(info["bytes"].sum())
    flops = float((info["flops_per_element"] * visited).sum())
    peak, peak_kind = measured_peak()
    hbm = {"bound": "hbm", "achieved": moved / total_s / 1e9, "peak": peak, "unit": "GB/s",
           "frac": moved / total_s / 1e9 / peak, "bytes_per_launch": moved / len(med),
           "avg_launch_ms": 1000 * total_s / len(med), "launches": int(pass_ms.size),
           "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback 6.8 TB/s"}  # fmt: skip
    arith = {"achieved": flops / total_s / 1e12, "unit": "TFLOP/s", "flops_per_evolution": flops}
    if real64 and fp64_peak:
        arith.update(bound="fp64", peak=fp64_peak, frac=flops / total_s / 1e12 / fp64_peak,
                     peak_source="measured: cuBLAS FP64 matmul 4096^3 on this GPU, best of 5")  # fmt: skip
    heaviest = max(per_pass, key=lambda p: p["ms"])
    return {"hbm": hbm, "arith": arith, "per_pass": per_pass, "heaviest_pass": heaviest, "evolve_ms": 1000 * total_s}


def _tune_summary(tune: dict | None) -> dict | None:
    """The autotuner's choice for the bench line: options, whether cached, candidate times."""
    if not tune:
        return None
    cands = [{**c["opts"], "ms": round(c["ms"], 3)} if "ms" in c else {**c["opts"], "error": c.get("error")}
             for c in tune.get("candidates", [])]  # fmt: skip
    return {"opts": tune.get("opts"), "cached": tune.get("cached"), "candidates_ms": cands}


def gb300_arm(args: argparse.Namespace) -> None:
    rank, world, local = dist_info()
    dist = Dist(world)
    import numpy as np
    import torch

    from lucivant_sim_gb300 import _lib, workloads as wl
    from lucivant_sim_gb300.batch import DensityBatch, run_density_batch

    _lib.set_device(local)
    torch.cuda.set_device(local)
    circuit, labels = workload()
    noises = wl.dm_noise_instances(args.instances, seed=SEED + rank)
    golden = load_golden() if rank == 0 else {}
    real64 = args.precision == "c128"  # the FP64 register: an FP64 roofline; df64 and c64: HBM
    fp64_peak = fp64_peak_tflops() if real64 and rank == 0 else None

    batch = DensityBatch(circuit, noises, precision=args.precision, autotune=not args.no_autotune)
    passes, real = batch.program.passes, batch.reg.real
    tune = batch.tune
    elem = {"c128": "double", "c64": "float", "df64": "lsg::DF"}[args.precision]
    kernel = f"k_tile_pipe<{elem}>" if real else f"k_tile_pipe<Cx<{elem}>>"
    specialized = batch.program.specialized
    if specialized:  # the passes run as kernels compiled for this circuit at run time
        kernel = f"lsg_pass_0..{passes - 1} (pipe_kernel specializations of {kernel})"
    stream = torch.cuda.ExternalStream(batch.reg.stream())
    run = timed_batch(batch, labels, args.steps, args.warmup, stream, local, dist)
    elapsed = run["elapsed"]
    cps = args.instances * args.steps * world / elapsed
    roof = pass_rooflines(batch, run["pass_ms"], real64, fp64_peak)
    moved_step = batch.bytes_per_evolve
    # reset, passes, expectations, probabilities (the Pauli-transfer register reduces every member
    # in one launch each; the complex form sums rows in a second launch and runs one per member)
    launches_per_step = 1 + passes + (2 if real else 2 + args.instances)
    accuracy = golden_errors(run["probs"], run["exps"], golden, noises)
    exps0, probs0 = run["exps"][:, :1].copy(), run["probs"][:1].copy()
    batch.free()

    # plain complex128 path on the same GPU: one instance at a time (instance 0), interpreted passes
    plain = DensityBatch(circuit, noises[:1], precision="c128")
    for _ in range(2):
        plain.evolve()
        plain.expectations(labels)
        p_ref = plain.probabilities()
    plain.reg.sync()
    reps = max(3, args.steps)
    t0 = time.perf_counter()
    for _ in range(reps):
        plain.evolve()
        e_ref = plain.expectations(labels)
        p_ref = plain.probabilities()
    plain.reg.sync()
    plain_s = (time.perf_counter() - t0) / reps
    plain.free()
    plain_cps = world / plain_s

    # and in Orrery's own form: the complex128 vectorised density matrix (superoperators on 2n bits)
    os.environ["LSG_DM_FORM"] = "superop"
    try:
        sup = DensityBatch(circuit, noises[:1], precision="c128")
    finally:
        del os.environ["LSG_DM_FORM"]
    for _ in range(2):
        sup.evolve()
        sup.expectations(labels)
        p_sup = sup.probabilities()
    sup.reg.sync()
    t0 = time.perf_counter()
    for _ in range(reps):
        sup.evolve()
        e_sup = sup.expectations(labels)
        p_sup = sup.probabilities()
    sup.reg.sync()
    sup_s = (time.perf_counter() - t0) / reps
    sup_form = sup.form
    sup.free()

    # the same instances in the other registers beside it: real32 (the complex64 request) and
    # double-float pairs (FP64-level accuracy from FP32 arithmetic)
    def beside(prec: str, dtype: str, what: str) -> dict:
        bx = DensityBatch(circuit, noises, precision=prec, autotune=not args.no_autotune)
        rx = timed_batch(bx, labels, args.steps, args.warmup, torch.cuda.ExternalStream(bx.reg.stream()), local, dist)
        roofx = pass_rooflines(bx, rx["pass_ms"], False, None)
        cpsx = args.instances * args.steps * world / rx["elapsed"]
        out = {
            "circuits_per_s": cpsx,
            "ms_per_step": 1000 * rx["elapsed"] / args.steps,
            "dtype": dtype,
            "register": what,
            "fused_passes": bx.program.passes,
            "autotune": _tune_summary(bx.tune),
            "speedup_vs_plain_c128": cpsx / plain_cps,
            "speedup_vs_plain_c128_superop": cpsx * sup_s / world,
            "speedup_vs_batched_headline": cpsx / cps,
            "roofline": dict(roofx["hbm"], kernel=f"lsg_pass_0..{bx.program.passes - 1} ({what})",
                             traffic=(lambda t: sum(t) / len(t) if t else None)(ncu_traffic(prec)),
                             heaviest_pass=roofx["heaviest_pass"], arith=roofx["arith"]),  # fmt: skip
            "per_pass": roofx["per_pass"],
            "accuracy_vs_orrery": golden_errors(rx["probs"], rx["exps"], golden, noises),
            "accuracy_vs_gpu_headline": {
                "probability_tvd": 0.5 * float(np.abs(rx["probs"][0] - probs0[0]).sum()),
                "max_probability_error": float(np.max(np.abs(rx["probs"][0] - probs0[0]))),
                "max_expectation_error": float(np.max(np.abs(rx["exps"][:, 0] - exps0[:, 0]))),
            },
            "clocks": rx["clocks"],
        }
        bx.free()
        return out

    c64 = beside("c64", "f32", "real32") if not args.no_c64 and real64 else None
    df64 = beside("df64", "f32 pairs (double-float)", "double-float pairs") if not args.no_c64 and real64 else None

    # end to end through the public batched API: host inputs in, host results out, every step
    e2e_steps = max(2, args.steps // 2)
    # one untimed call: the halves the call evolves are programs of their own shape (specialized
    # passes compiled once per process, like the whole batch's above)
    run_density_batch(circuit, noises, labels, precision=args.precision, autotune=not args.no_autotune)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        probs_h, exps_h = run_density_batch(circuit, noises, labels, precision=args.precision,
                                            autotune=not args.no_autotune)
    e2e_s = dist.max((time.perf_counter() - t0) / e2e_steps)
    # operator tables and data pools (one per half the call evolves), Pauli masks
    h2d = int(e2e_upload_bytes(circuit, noises) + 2 * 8 * len(labels))
    d2h = int(probs_h.nbytes + exps_h.nbytes)

    if rank == 0:
        tr = ncu_traffic({"c128": "f64"}.get(args.precision, args.precision))
        traffic = sum(tr) / len(tr) if tr else None  # mean DRAM bytes per full-size launch (ncu)
        if real64:
            roofline = dict(roof["arith"], kernel=kernel, traffic=traffic, hbm=roof["hbm"],
                            heaviest_pass=roof["heaviest_pass"])  # fmt: skip
        else:
            roofline = dict(roof["hbm"], kernel=kernel, traffic=traffic, arith=roof["arith"],
                            heaviest_pass=roof["heaviest_pass"])  # fmt: skip
        roofline["traffic_source"] = (f"profiles/tile_pass_dm12_{({'c128': 'f64'}).get(args.precision, args.precision)}.md: ncu DRAM read+write "
                                      "of an 8-instance capture x 32, per launch, mean over the passes")
        line = {
            "metric": "circuits/s",
            "value": cps,
            "unit": "circuits/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": 1000 * elapsed / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": {"c128": "f64", "c64": "f32", "df64": "f32 pairs (double-float)"}[args.precision],
            "data": "synthetic",
            "config": dict(config_block(args), form=batch.form),
            "hbm_gbs_moved": moved_step * args.steps * world / elapsed / 1e9,
            "fused_passes": passes,
            "specialized_passes": specialized,
            "autotune": _tune_summary(tune),
            "accuracy_vs_orrery": accuracy,
            "plain_c128": {
                "circuits_per_s": plain_cps,
                "ms_per_circuit": 1000 * plain_s,
                "speedup_of_batched": cps / plain_cps,
                "what": "one instance (instance 0) per run, real64 Pauli-transfer register, interpreted passes",
                "probability_max_abs_vs_batched": float(np.max(np.abs(p_ref[0] - probs0[0]))),
                "expectation_max_abs_vs_batched": float(np.max(np.abs(e_ref[:, 0] - exps0[:, 0]))),
            },
            "plain_c128_superop": {
                "circuits_per_s": world / sup_s,
                "ms_per_circuit": 1000 * sup_s,
                "speedup_of_batched": cps * sup_s / world,
                "what": f"one instance (instance 0) per run, complex128 vectorised density matrix ({sup_form}: "
                        "Orrery's form), interpreted passes",
                "probability_max_abs_vs_batched": float(np.max(np.abs(p_sup[0] - probs0[0]))),
                "expectation_max_abs_vs_batched": float(np.max(np.abs(e_sup[:, 0] - exps0[:, 0]))),
            },
            "roofline": roofline,
            "per_pass": roof["per_pass"],
            "c64_batched": c64,
            "df64_batched": df64,
            "e2e": {
                "value": args.instances * world / e2e_s,
                "unit": "circuits/s",
                "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "api": "lucivant_sim_gb300.batch.run_density_batch",
            },
            "gpu_launches": launches_per_step * args.steps,
            "clocks": run["clocks"],
        }
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline()
        print(json.dumps(line, default=_plain), flush=True)
    dist.close()


# ------------------------------------------------------------------------------ served mix


def _circuits(job: dict) -> int:
    return len(job["params"]) if job["kind"] == "expect" else 1


def _plain_c128(job: dict):
    """One job through the direct API at complex128, one circuit at a time."""
    import lucivant_sim_gb300 as ls
    from lucivant_sim_gb300 import serve

    if job["kind"] == "expect":
        return [ls.expectation(ls.parse(job["qasm"], p), job["observable"], precision="c128") for p in job["params"]]
    noise = ls.NoiseModel.uniform(**serve.DEFAULT_NOISE) if job["kind"] == "density" else None
    return ls.run(job["qasm"], shots=job["shots"], seed=job["seed"], noise=noise, precision="c128").counts


def serve_arm(args: argparse.Namespace) -> None:
    """The served mix on one GPU: offered at ``--rate`` jobs/s for p50/p99 latency, then all at
    once for throughput; the same jobs run one at a time through the direct complex128 API for
    the plain rate, and the complex64 results are checked against complex128."""
    rank, world, local = dist_info()
    if rank != 0:
        return
    import numpy as np

    import lucivant_sim_gb300 as ls
    from lucivant_sim_gb300 import _lib, serve, workloads as wl

    _lib.set_device(local)
    jobs = wl.served_mix(args.jobs, rate=args.rate, seed=5)
    warm = wl.served_mix(max(args.warmup, 3) * 8, rate=args.rate, seed=99)
    circuits = sum(_circuits(j) for j in jobs)
    prec = "c64"  # the served path runs complex64 states
    with serve.Server(precision=prec, workers=args.serve_workers) as srv:
        serve.replay(warm, srv, realtime=False)
        clocks = Clocks(local)
        clocks.start()
        burst = serve.replay(jobs, srv, realtime=False)  # all at once: throughput
        offered = serve.replay(jobs, srv, realtime=True)  # at the offered rate
        # at 70% of the measured throughput: latency without a growing queue
        sustainable = 0.7 * len(jobs) / burst["elapsed_s"]
        steady_jobs = wl.served_mix(args.jobs, rate=sustainable, seed=6)
        steady = serve.replay(steady_jobs, srv, realtime=True)
        clock_info = clocks.stop()
    # plain complex128, one job at a time, on a bounded prefix of the same mix
    sample = jobs[: max(8, min(len(jobs), 60))]
    _plain_c128(sample[0])
    t0 = time.perf_counter()
    plain = [_plain_c128(j) for j in sample]
    plain_s = time.perf_counter() - t0
    plain_cps = sum(_circuits(j) for j in sample) / plain_s
    # complex64 accuracy against complex128 on the prefix
    tvd, exp_err, same_counts = 0.0, 0.0, 0
    for job, res, ref in zip(sample, burst["results"], plain, strict=False):
        if job["kind"] == "expect":
            exp_err = max(exp_err, float(np.max(np.abs(np.asarray(res["values"]) - np.asarray(ref)))))
        else:
            same_counts += int(res["counts"] == ref)
            if job["kind"] == "sample" and job["width"] <= 20:
                c = ls.parse(job["qasm"])
                p64 = ls.probabilities_array(c, precision="c64")
                p128 = ls.probabilities_array(c, precision="c128")
                tvd = max(tvd, 0.5 * float(np.abs(p64 - p128).sum()))
    cps = circuits / burst["elapsed_s"]
    line = {
        "metric": "served circuits/s",
        "value": cps,
        "unit": "circuits/s",
        "n_gpus": 1,
        "steps": 1,
        "warmup": len(warm),
        "ms_per_step": 1000 * burst["elapsed_s"],
        "higher_is_better": True,
        "scaling": "replicas only",
        "vs_baseline": None,
        "dtype": prec,
        "data": "synthetic",
        "config": {
            "workload": f"served mix: {args.jobs} jobs ({circuits} circuits), widths 8..26, depths 10..100, "
            "30% 8-point HEA sweeps with 20-term Pauli sums, 20% noisy density matrices, 50% sampled (1000 shots)",
            "precision": prec,
            "offered_rate_jobs_per_s": args.rate,
            "worker_slots": args.serve_workers,
        },
        "latency_at_offered_rate": {"p50_s": offered["p50_s"], "p99_s": offered["p99_s"],
                                    "circuits_per_s": circuits / offered["elapsed_s"],
                                    "note": "above the sustainable rate the queue grows through the run"},
        "latency_at_70pct_of_throughput": {"rate_jobs_per_s": sustainable, "p50_s": steady["p50_s"],
                                           "p99_s": steady["p99_s"]},  # fmt: skip
        "latency_all_at_once": {"p50_s": burst["p50_s"], "p99_s": burst["p99_s"]},
        "phases_at_offered_rate": offered["phases"],
        "phases_at_70pct_of_throughput": steady["phases"],
        "plain_c128": {"circuits_per_s": plain_cps, "jobs_timed": len(sample), "speedup_of_served": cps / plain_cps},
        "accuracy": {"max_probability_tvd_vs_c128": tvd, "max_expectation_error_vs_c128": exp_err,
                     "counts_identical_to_c128": f"{same_counts} of {sum(j['kind'] != 'expect' for j in sample)}"},  # fmt: skip
        "clocks": clock_info,
    }
    print(json.dumps(line, default=_plain), flush=True)


# ------------------------------------------------------------------------------ other configurations


def _line(metric: str, value: float, unit: str, workload: str, dtype: str, **extra) -> None:
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "higher_is_better": True,
            "scaling": "replicas only", "vs_baseline": None, "dtype": dtype, "data": "synthetic",
            "config": {"workload": workload}}  # fmt: skip
    line.update(extra)
    print(json.dumps(line, default=_plain), flush=True)


def sv_arm(args: argparse.Namespace) -> None:
    """Config 1: 20-qubit, 20-layer brickwork statevector, 10,000 shots, seed 7, through ls.run."""
    import numpy as np

    import lucivant_sim_gb300 as ls
    from lucivant_sim_gb300 import _lib, engine, qasm, workloads as wl

    _lib.set_device(dist_info()[2])
    c = qasm.parse(wl.brickwork(20, 20, seed=7))
    out = {}
    for prec in ("c128", "c64"):
        code = engine.precision_code(prec)
        reg = _lib.Register(20, code, 1)
        prog = _lib.Program(reg, engine.sv_oplist(c))
        for _ in range(max(args.warmup, 3)):
            prog.run_timed(reg)
        t = np.array([prog.run_timed(reg).sum() for _ in range(args.steps)])
        passes, ms = prog.passes, float(np.median(t))
        prog.free()
        reg.free()
        for _ in range(2):
            ls.run(c, shots=10_000, seed=7, precision=prec)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            r = ls.run(c, shots=10_000, seed=7, precision=prec)
        run_s = (time.perf_counter() - t0) / args.steps
        out[prec] = {"passes": passes, "evolve_ms": ms, "pass_gbs": 2 * (_lib.ELEM_BYTES[code] << 20) * passes / ms / 1e6,
                     "run_ms": 1000 * run_s, "circuits_per_s": 1 / run_s, "counts_distinct": len(r.counts)}  # fmt: skip
    _line("statevector circuits/s (ls.run, 10,000 shots)", out["c128"]["circuits_per_s"], "circuits/s",
          "statevector 20q x 20 brickwork layers, 10,000 shots, seed 7 (16 MiB c128 state: L2-resident, "
          "no HBM-fraction claim)", "c128", steps=args.steps, by_precision=out)  # fmt: skip


def traj_arm(args: argparse.Namespace) -> None:
    """Config 3: 18 qubits, 16 rounds with mid-circuit measurement, 4096 shots; batched complex64
    (every shot a register member) and serial complex128 (Orrery's draw order) on a sample."""
    import lucivant_sim_gb300 as ls
    from lucivant_sim_gb300 import _lib, qasm, workloads as wl

    _lib.set_device(dist_info()[2])
    c = qasm.parse(wl.midcircuit(18, 16, seed=7))
    noise = ls.NoiseModel.uniform(single=1e-3, two=1e-2)
    ls.run(c, shots=64, seed=1, noise=noise, method="trajectories", precision="c64", trajectory_mode="batched")
    t0 = time.perf_counter()
    rb = ls.run(c, shots=4096, seed=7, noise=noise, method="trajectories", precision="c64", trajectory_mode="batched")
    batched_s = time.perf_counter() - t0
    serial_shots = 256
    ls.run(c, shots=8, seed=1, noise=noise, method="trajectories", precision="c128", trajectory_mode="serial")
    t0 = time.perf_counter()
    ls.run(c, shots=serial_shots, seed=7, noise=noise, method="trajectories", precision="c128", trajectory_mode="serial")
    serial_s = time.perf_counter() - t0
    _line("trajectory shots/s", 4096 / batched_s, "shots/s",
          "trajectories 18q x 16 rounds (measure 4, conditional x, reset), depolarising 1e-3/1e-2, 4096 shots",
          "c64", batched={"shots": 4096, "seconds": batched_s, "distinct_outcomes": len(rb.counts)},
          serial_c128={"shots": serial_shots, "seconds": serial_s, "shots_per_s": serial_shots / serial_s,
                       "note": "Orrery's draw order; identical counts to the reference for the same seed"})  # fmt: skip


def stab_arm(args: argparse.Namespace) -> None:
    """Config 4: 2048-qubit Clifford layers with Pauli noise, 1000 shots, seed 11 (Pauli frames)."""
    import numpy as np

    from lucivant_sim_gb300 import _lib, stabilizer, workloads as wl

    _lib.set_device(dist_info()[2])
    layers = 1000
    c = wl.clifford_layers_circuit(2048, layers, seed=11)
    noise = wl.stabilizer_noise(1e-3)
    small = wl.clifford_layers_circuit(2048, 10, seed=11)
    stabilizer.run_counts(small, 100, noise, np.random.default_rng(11))
    t0 = time.perf_counter()
    tally = stabilizer.run_counts(c, 1000, noise, np.random.default_rng(11))
    s = time.perf_counter() - t0
    gates = sum(1 for op in c.operations if op.kind == "gate")
    _line("stabilizer gate-shots/s", gates * 1000 / s, "gate-shots/s",
          "stabilizer 2048q x 1000 layers (h/s/sdg/x/z + cx, cz on a random matching), depolarising 1e-3, "
          "readout 0.01/0.03, 1000 shots, seed 11", "uint32 bit-packed",
          seconds=s, gates=gates, layers_per_s=layers / s, distinct_outcomes=len(tally))  # fmt: skip


def main() -> None:
    args = parse_args()
    if args.impl == "reference":
        reference_arm(args)
    elif args.workload == "serve":
        serve_arm(args)
    elif args.workload == "sv20":
        sv_arm(args)
    elif args.workload == "traj18":
        traj_arm(args)
    elif args.workload == "stab2048":
        stab_arm(args)
    else:
        gb300_arm(args)


if __name__ == "__main__":
    main()
