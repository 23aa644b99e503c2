#!/usr/bin/env python3
"""Benchmark: the batched noisy density-matrix hot path on one GB300 (per rank).

Workload (one step): 256 noise instances of a 12-qubit, 12-layer u3+cx brickwork circuit (angles
U[0, 2π) from seed 7), each with thermal relaxation (T1 = 120, T2 = 90, t = 0.05) composed with a
depolarising one-qubit error ~ U[1e-4, 5e-3] on every u3, depolarising two-qubit error
~ U[1e-3, 3e-2] on every cx, evolved as one 256-member register of density matrices in the
Pauli-transfer form (24-bit registers of real32 coefficients for the complex64 request, 16 GiB),
from |0><0| through passes compiled for the circuit at run time, then the exact probabilities and
the 23 observables <Z_i>, <Z_i Z_i+1> of every instance. Inputs are larger than L2 (no flush
needed).

metric: statevector HBM GB/s — algorithmic HBM bytes of the step (2 x register bytes per fused
pass, one register write to reset, the reduction reads) per second, whole job; the passes skip
tiles the circuit has not reached yet, and the roofline counts the bytes they move. Beside it:
the instances (circuits) per second, the end-to-end rate through the public batched call, and the
same circuit as a plain complex128 single-instance run on the same GPU ("plain_c128"), with the
complex64 path's error against it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun each rank runs its own 256 instances on its own GPU (weak scaling, no data-path
collective). ``--impl reference`` times the CPU port of Orrery's algorithm (the oracle) on the
host cores instead, on rank 0 only.
"""

from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

QUBITS, LAYERS, SEED, INSTANCES = 12, 12, 7, 256
FALLBACK_HBM_GBS = 6800.0
CPU_SAMPLE_U3, CPU_SAMPLE_CX = 4, 2  # oracle ops timed for the CPU baseline (about 10-15 s)
REF_SAMPLE_U3, REF_SAMPLE_CX = 2, 1  # per worker per step in the reference arm


def parse_args() -> argparse.Namespace:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--precision", choices=("c64", "c128"), default="c64")
    ap.add_argument("--instances", type=int, default=INSTANCES)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", choices=("dm-batch", "serve", "sv20", "traj18", "stab2048"), default="dm-batch",
                    help="dm-batch: the batched density-matrix step (default); serve: the served mix; sv20: "
                    "statevector 20q x 20 layers; traj18: trajectories 18q x 16 rounds x 4096 shots; stab2048: "
                    "stabilizer 2048q x 1000 layers x 1000 shots")  # fmt: skip
    ap.add_argument("--jobs", type=int, default=400, help="serve: jobs in the served mix")
    ap.add_argument("--rate", type=float, default=200.0, help="serve: offered arrivals per second")
    return ap.parse_args()


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
        "clocks_event_reasons.sw_power_cap"
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
        sm, smax, reasons = [], [], set()
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
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


def measured_peak() -> tuple[float, str]:
    path = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(path.read_text())["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(precision: str) -> float | None:
    """DRAM bytes per launch of the tile pass, from the committed ncu summary (scaled there to a
    full-size launch), or None."""
    path = ROOT / "profiles" / f"tile_pass_dm12_{precision}.md"
    if not path.exists():
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", path.read_text())
    return float(m.group(1)) if m else None


def workload():
    from lucivant_sim_gb300 import qasm, workloads as wl

    circuit = qasm.parse(wl.brickwork(QUBITS, LAYERS, seed=SEED, measure=False))
    return circuit, wl.z_observables(QUBITS)


def bytes_per_instance(circuit, noises, precision: str) -> tuple[int, int]:
    """(algorithmic HBM bytes per instance, fused passes) for one evolution plus reductions."""
    from lucivant_sim_gb300 import _lib, engine

    code = engine.precision_code(precision)
    if engine.dm_form(circuit, noises[:1]) == "ptm":
        code = engine.REAL_OF[code]
        ops = engine.ptm_oplist(circuit, noises[:1])
        reads = (1 << QUBITS) + 23  # the diagonal Paulis (probabilities), one coefficient per Z term
    else:
        ops = engine.dm_oplist(circuit, noises[:1])
        reads = 24 << QUBITS  # the diagonal, read by probabilities and by each of the 23 Z terms
    passes = _lib.plan_passes(2 * QUBITS, code, ops)
    elt = _lib.ELEM_BYTES[code]
    member = elt << (2 * QUBITS)
    # 2 x member per pass, 1 x member to reset, and the reduction reads
    return 2 * member * passes + member + reads * elt, passes


# ------------------------------------------------------------------------------ CPU legs


def _oracle_sample(args: tuple[int, int, int]) -> tuple[float, float]:
    """Time the oracle on the first u3 and cx gate+channel operations of one instance; returns
    the seconds per u3 operation and per cx operation."""
    n_u3, n_cx, instance = args
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    import numpy as np

    from lucivant_sim_gb300 import workloads as wl
    from oracle import dense

    circuit, _ = workload()
    noise = wl.dm_noise_instances(INSTANCES, seed=SEED)[instance % INSTANCES]
    n = QUBITS
    rho = np.zeros(1 << (2 * n), dtype=np.complex128)
    rho[0] = 1
    gates = [op for op in circuit.operations if op.kind == "gate"]
    u3 = [g for g in gates if len(g.qubits) == 1][:n_u3]
    cx = [g for g in gates if len(g.qubits) == 2][:n_cx]
    times = []
    for group in (u3, cx):
        t0 = time.perf_counter()
        for op in group:
            rho = dense.apply_bits(rho, 2 * n, op.matrix, [n + q for q in op.qubits])
            rho = dense.apply_bits(rho, 2 * n, op.matrix.conj(), list(op.qubits))
            ch = noise.gate_error(op.name, op.qubits)
            if ch is not None:
                rho = dense.dm_channel(rho, n, ch, op.qubits)
        times.append((time.perf_counter() - t0) / max(len(group), 1))
    return times[0], times[1]


def _project(t_u3: float, t_cx: float, circuit) -> float:
    gates = [op for op in circuit.operations if op.kind == "gate"]
    n1 = sum(1 for g in gates if len(g.qubits) == 1)
    return n1 * t_u3 + (len(gates) - n1) * t_cx


def cpu_baseline(circuit, bytes_inst: int) -> dict:
    """The oracle (a port of Orrery's algorithm) on one host thread, on a bounded sample."""
    code = (
        "import sys, json; sys.path.insert(0, %r); import bench; "
        "print(json.dumps(bench._oracle_sample((%d, %d, 0))))" % (str(ROOT), CPU_SAMPLE_U3, CPU_SAMPLE_CX)
    )
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1")
    t0 = time.perf_counter()
    proc = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=600)
    wall = time.perf_counter() - t0
    if proc.returncode != 0:
        return {"value": None, "unit": "GB/s", "error": proc.stderr.strip()[-300:]}
    t_u3, t_cx = json.loads(proc.stdout.strip().splitlines()[-1])
    per_circuit = _project(t_u3, t_cx, circuit)
    return {
        "value": bytes_inst / per_circuit / 1e9,
        "unit": "GB/s",
        "cores": 1,
        "kind": "port",
        "sample": f"oracle density-matrix evolution of instance 0: first {CPU_SAMPLE_U3} u3 and {CPU_SAMPLE_CX} cx "
        f"gate+channel ops timed ({wall:.1f} s wall), projected to the full circuit "
        f"({per_circuit:.1f} s per instance, {1 / per_circuit:.4f} circuits/s)",
        "circuits_per_s": 1 / per_circuit,
    }


def reference_arm(args: argparse.Namespace) -> None:
    rank, world, _ = dist_info()
    if rank != 0:
        return
    import multiprocessing as mp

    circuit, _ = workload()
    from lucivant_sim_gb300 import workloads as wl

    noises = wl.dm_noise_instances(INSTANCES, seed=SEED)
    bytes_inst, _ = bytes_per_instance(circuit, noises, args.precision)
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    os.environ["OPENBLAS_NUM_THREADS"] = "1"  # inherited by the spawned workers: one thread each
    with ctx.Pool(cores) as pool:
        jobs = [(REF_SAMPLE_U3, REF_SAMPLE_CX, i) for i in range(cores)]
        for _ in range(args.warmup):
            pool.map(_oracle_sample, jobs)
        per_step, circuits = [], 0.0
        for _ in range(args.steps):
            t0 = time.perf_counter()
            res = pool.map(_oracle_sample, jobs)
            dt = time.perf_counter() - t0
            # each worker did a fraction of one circuit: fraction = sampled time / projected time
            frac = sum((REF_SAMPLE_U3 * a + REF_SAMPLE_CX * b) / _project(a, b, circuit) for a, b in res)
            circuits += frac
            per_step.append(dt)
    elapsed = sum(per_step)
    cps = circuits / elapsed
    value = cps * bytes_inst / 1e9
    line = {
        "impl": "reference",
        "metric": "statevector HBM GB/s",
        "value": value,
        "unit": "GB/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1000 * elapsed / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "c128",
        "data": "synthetic",
        "config": config_block(args),
        "circuits_per_s": cps,
        "cpu_baseline": {
            "value": value,
            "unit": "GB/s",
            "cores": cores,
            "kind": "port",
            "sample": f"each step: {cores} processes, each evolving the first {REF_SAMPLE_U3} u3 and {REF_SAMPLE_CX} cx "
            "gate+channel ops of one instance with the oracle; circuits = sampled fraction of the full circuit",
        },
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def config_block(args: argparse.Namespace) -> dict:
    return {
        "workload": f"density_matrix {QUBITS}q x {LAYERS} brickwork layers, {args.instances} noise instances per GPU",
        "qubits": QUBITS,
        "layers": LAYERS,
        "instances_per_gpu": args.instances,
        "precision": args.precision,
        "noise": "thermal_relaxation(120, 90, 0.05) composed with depolarising U[1e-4,5e-3] on u3; "
        "depolarising U[1e-3,3e-2] on cx; readout 2e-2",
        "outputs": "probabilities (2^12) and 23 Z observables per instance",
        # the workload's gates act on at most two qubits: the Pauli-transfer form, real32 for a
        # complex64 request (real64 for complex128)
        "form": "ptm",
        "l2": f"register {((4 if args.precision == 'c64' else 8) * args.instances << 24) / 2**30:.0f} GiB > L2: no flush",
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
    bytes_inst, passes = bytes_per_instance(circuit, noises, args.precision)
    bytes_step = bytes_inst * args.instances

    batch = DensityBatch(circuit, noises, precision=args.precision)
    assert batch.program.passes == passes
    form, upload_bytes, reg_bytes = batch.form, batch.upload_bytes, batch.register_bytes
    real = batch.reg.real
    kernel = f"k_tile_pipe<{'float' if args.precision == 'c64' else 'double'}>" if real else \
        f"k_tile_pipe<Cx<{'float' if args.precision == 'c64' else 'double'}>>"
    specialized = batch.program.specialized
    if specialized:  # the passes run as kernels compiled for this circuit at run time
        kernel = f"lsg_pass_0..{passes - 1} (pipe_kernel specializations of {kernel})"
    stream = torch.cuda.ExternalStream(batch.reg.stream())

    def step(timed: list | None = None) -> tuple:
        if timed is None:
            batch.evolve()
        else:
            timed.append(batch.evolve_timed())
        return batch.expectations(labels), batch.probabilities()

    for _ in range(args.warmup):
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
    for _ in range(args.steps):
        exps, probs = step(pass_ms)
    t_end.record(stream)
    t_end.synchronize()
    batch.reg.sync()
    clock_info = clocks.stop()
    dist.barrier()
    elapsed = dist.max(t_start.elapsed_time(t_end) / 1000.0)
    value = bytes_step * args.steps * world / elapsed / 1e9
    cps = args.instances * args.steps * world / elapsed
    # reset, passes, expectations, probabilities (the Pauli-transfer register reduces every member
    # in one launch each; the complex form sums rows in a second launch and runs one per member)
    launches_per_step = 1 + passes + (2 if real else 2 + args.instances)

    all_pass = np.concatenate(pass_ms)
    avg_launch_s = float(all_pass.mean()) / 1000.0
    # bytes the passes actually move: a run from |0><0| skips tiles the circuit has not reached
    # (still zero), so early passes move less than 2 x register bytes
    nominal_launch_bytes = 2 * batch.register_bytes
    moved_per_run = batch.bytes_per_evolve
    launch_bytes = moved_per_run / passes
    peak, peak_kind = measured_peak()
    achieved = launch_bytes / avg_launch_s / 1e9
    traffic = ncu_traffic(args.precision)
    roofline = {
        "kernel": kernel,
        "bound": "hbm",
        "achieved": achieved,
        "peak": peak,
        "unit": "GB/s",
        "frac": achieved / peak,
        "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback 6.8 TB/s",
        "traffic": traffic,
        "bytes_per_launch": launch_bytes,
        "nominal_bytes_per_launch": nominal_launch_bytes,
        "skipped_zero_tile_bytes_frac": 1.0 - moved_per_run / (nominal_launch_bytes * passes),
        "avg_launch_ms": avg_launch_s * 1000,
        "launches": int(all_pass.size),
        "share_of_step": float(all_pass.sum()) / 1000.0 / (elapsed / 1.0) if world == 1 else None,
    }

    # plain complex128 path on the same GPU: one instance at a time (instance 0)
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
    tvd = 0.5 * float(np.abs(probs[0] - p_ref[0]).sum())
    exp_err = float(np.max(np.abs(exps[:, 0] - e_ref[:, 0])))

    # end to end through the public batched API: host inputs in, host results out, every step
    e2e_steps = max(2, args.steps // 2)
    batch.free()
    # one untimed call: the halves the call evolves are programs of their own shape (specialized
    # passes compiled once per process, like the whole batch's above)
    run_density_batch(circuit, noises, labels, precision=args.precision)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        probs_h, exps_h = run_density_batch(circuit, noises, labels, precision=args.precision)
    e2e_s = dist.max((time.perf_counter() - t0) / e2e_steps)
    from lucivant_sim_gb300 import engine

    # operator tables and data pools (one per half the call evolves), Pauli masks
    h2d = int(e2e_upload_bytes(circuit, noises) + 2 * 8 * len(labels))
    d2h = int(probs_h.nbytes + exps_h.nbytes)

    if rank == 0:
        line = {
            "metric": "statevector HBM GB/s",
            "value": value,
            "unit": "GB/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": 1000 * elapsed / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": ("f32" if args.precision == "c64" else "f64") if real else args.precision,
            "data": "synthetic",
            "config": dict(config_block(args), form=form),
            "circuits_per_s": cps,
            "fused_passes": passes,
            "specialized_passes": specialized,
            "plain_c128": {
                "circuits_per_s": world / plain_s,
                "ms_per_circuit": 1000 * plain_s,
                "speedup_of_batched": cps / (world / plain_s),
            },
            "accuracy": {"probability_tvd_vs_c128": tvd, "max_expectation_error_vs_c128": exp_err},
            "roofline": roofline,
            "e2e": {
                "value": bytes_step * world / e2e_s / 1e9,
                "unit": "GB/s",
                "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "circuits_per_s": args.instances * world / e2e_s,
                "api": "lucivant_sim_gb300.batch.run_density_batch",
            },
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clock_info,
        }
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(circuit, bytes_inst)
        print(json.dumps(line), flush=True)
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
    with serve.Server(precision=args.precision) as srv:
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
        "dtype": args.precision,
        "data": "synthetic",
        "config": {
            "workload": f"served mix: {args.jobs} jobs ({circuits} circuits), widths 8..26, depths 10..100, "
            "30% 8-point HEA sweeps with 20-term Pauli sums, 20% noisy density matrices, 50% sampled (1000 shots)",
            "precision": args.precision,
            "offered_rate_jobs_per_s": args.rate,
        },
        "latency_at_offered_rate": {"p50_s": offered["p50_s"], "p99_s": offered["p99_s"],
                                    "circuits_per_s": circuits / offered["elapsed_s"],
                                    "note": "above the sustainable rate the queue grows through the run"},
        "latency_at_70pct_of_throughput": {"rate_jobs_per_s": sustainable, "p50_s": steady["p50_s"],
                                           "p99_s": steady["p99_s"]},  # fmt: skip
        "latency_all_at_once": {"p50_s": burst["p50_s"], "p99_s": burst["p99_s"]},
        "plain_c128": {"circuits_per_s": plain_cps, "jobs_timed": len(sample), "speedup_of_served": cps / plain_cps},
        "accuracy": {"max_probability_tvd_vs_c128": tvd, "max_expectation_error_vs_c128": exp_err,
                     "counts_identical_to_c128": f"{same_counts} of {sum(j['kind'] != 'expect' for j in sample)}"},  # fmt: skip
        "clocks": clock_info,
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------ other configurations


def _line(metric: str, value: float, unit: str, workload: str, dtype: str, **extra) -> None:
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "higher_is_better": True,
            "scaling": "replicas only", "vs_baseline": None, "dtype": dtype, "data": "synthetic",
            "config": {"workload": workload}}  # fmt: skip
    line.update(extra)
    print(json.dumps(line), flush=True)


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
