"""The serving loop: a job's result inside a concurrent mix is identical to the same job run
alone, and the served complex64 results agree with complex128 (counts identical for shared
seeds unless a shot lies on a CDF boundary, expectations to 1e-5)."""

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
