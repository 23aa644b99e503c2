"""The serving loop: a job's result inside a concurrent mix is identical to the same job run
alone; the served complex64 results agree with the direct API (identical counts) and with the
oracle's complex128 results (expectations to 1e-5; counts identical except for shots whose
uniform lies within 4e-6 of a CDF entry, each moving one count)."""

from __future__ import annotations

import numpy as np
import pytest

import lucivant_sim_gb300 as ls
from lucivant_sim_gb300 import _lib, serve, workloads as wl
from oracle import dense

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mix():
    return wl.served_mix(48, seed=21, widths=(6, 14), depths=(4, 30), shots=500, sweep=4)


def _same(a: dict, b: dict) -> bool:
    if "values" in a:
        return np.array_equal(a["values"], b["values"])
    return a["counts"] == b["counts"]


def test_alone_equals_mix(mix):
    alone = [serve.execute(serve.prepare(dict(j, id=i)), _lib.C64) for i, j in enumerate(mix)]
    with serve.Server(precision="c64", workers=6, prep_workers=4) as srv:
        out = serve.replay(mix, srv, realtime=False)
    assert len(out["results"]) == len(mix)
    for a, b in zip(alone, out["results"], strict=True):
        assert _same(a, b)
    assert 0 < out["p50_s"] <= out["p99_s"]


def test_served_results_match_the_direct_api(mix):
    with serve.Server(precision="c64", workers=4, prep_workers=2) as srv:
        out = serve.replay(mix[:16], srv, realtime=False)
    for job, res in zip(mix[:16], out["results"], strict=True):
        if job["kind"] == "expect":
            for b, params in enumerate(job["params"]):
                c = ls.parse(job["qasm"], params)
                want = dense.expectation(c, job["observable"])
                assert abs(res["values"][b] - want) < 1e-5
        elif job["kind"] == "sample":
            direct = ls.run(job["qasm"], shots=job["shots"], seed=job["seed"], precision="c64")
            assert res["counts"] == direct.counts
        else:
            noise = ls.NoiseModel.uniform(**serve.DEFAULT_NOISE)
            direct = ls.run(job["qasm"], shots=job["shots"], seed=job["seed"], noise=noise, precision="c64")
            assert res["counts"] == direct.counts


def test_jobs_too_large_for_the_budget_are_refused():
    with serve.Server(precision="c64", workers=2, prep_workers=1, memory_bytes=1 << 20) as srv:
        fut = srv.submit(dict(kind="sample", qasm=wl.brickwork(20, 2, seed=1), shots=10, seed=1))
        with pytest.raises(MemoryError, match="admits at most"):
            fut.result(timeout=120)


def test_jobs_of_one_structure_run_together_with_the_results_they_get_alone():
    """Sampled and noisy jobs of one width and depth (other angles, seeds) queued behind one
    worker are grouped into one register; every grouped job's counts equal its counts alone."""
    jobs = []
    for s in range(6):
        jobs.append(dict(kind="sample", arrival=0.0, qasm=wl.brickwork(9, 6, seed=100 + s), shots=700, seed=s, width=9))
        jobs.append(dict(kind="density", arrival=0.0, qasm=wl.brickwork(5, 4, seed=200 + s), shots=700, seed=s, width=5))
    jobs += [dict(j, id=i) for i, j in enumerate(wl.served_mix(6, seed=3, widths=(6, 10), depths=(4, 12), shots=300, sweep=3))]
    alone = [serve.execute(serve.prepare(dict(j, id=i)), _lib.C64) for i, j in enumerate(jobs)]
    with serve.Server(precision="c64", workers=1, prep_workers=2, group_max=8) as srv:
        out = serve.replay(jobs, srv, realtime=False)
    grouped = [r for r in out["results"] if r.get("batched_with", 1) > 1]
    assert grouped, "no jobs were grouped"
    for a, b in zip(alone, out["results"], strict=True):
        assert _same(a, b)


def _oracle_cdf(circuit, probs: np.ndarray, shots: int, seed: int, eps: float) -> tuple[np.ndarray, np.ndarray]:
    """The oracle's CDF index of every shot (the run's first ``shots`` uniforms of
    ``default_rng(seed)``) and which shots lie within ``eps`` of a CDF entry."""
    measured = sorted({q for q, _ in circuit.final_measurements()})
    cum = np.cumsum(dense.marginal(probs, circuit.num_qubits, measured))
    cum /= cum[-1]
    u = np.random.default_rng(seed).random(shots)
    idx = np.searchsorted(cum, u, side="right")
    below = np.where(idx > 0, cum[np.maximum(idx - 1, 0)], 0.0)
    above = cum[np.minimum(idx, cum.size - 1)]
    return idx, (u - below < eps) | (above - u < eps)


def test_served_counts_against_the_oracle(mix):
    """Served complex64 statevector jobs and real32 Pauli-transfer density jobs against the
    oracle's complex128 counts for the same seeds. The served probabilities lie within 1e-6 TVD of
    the oracle's, so each CDF entry (normalised) moves by less than 4e-6: every count difference
    must come from a shot whose uniform lies that close to a CDF entry, each such shot moving one
    count (for statevector jobs, to a neighbouring outcome in CDF order)."""
    eps = 4e-6
    jobs = [j for j in mix if j["kind"] in ("sample", "density")]
    assert len(jobs) >= 10
    with serve.Server(precision="c64", workers=4, prep_workers=2) as srv:
        out = serve.replay(jobs, srv, realtime=False)
    exact = 0
    for job, res in zip(jobs, out["results"], strict=True):
        c = ls.parse(job["qasm"])
        noise = ls.NoiseModel.uniform(**serve.DEFAULT_NOISE) if job["kind"] == "density" else None
        want, _, _ = dense.run_counts(c, job["shots"], job["seed"], noise)
        idx, near = _oracle_cdf(c, dense.probabilities_array(c, noise), job["shots"], job["seed"], eps)
        got = res["counts"]
        diff = {k for k in set(want) | set(got) if want.get(k) != got.get(k)}
        moved = sum(abs(want.get(k, 0) - got.get(k, 0)) for k in diff)
        assert moved <= 2 * int(near.sum()), (job["kind"], job["width"], moved, int(near.sum()))
        if job["kind"] == "sample":  # every qubit measured in order: the outcome read as binary is the CDF index
            allowed = {int(idx[s]) + d for s in np.flatnonzero(near) for d in (-1, 0, 1)}
            assert {int(k, 2) for k in diff} <= allowed, (job["width"], sorted(diff)[:6])
        exact += not diff
    assert exact >= len(jobs) // 2
