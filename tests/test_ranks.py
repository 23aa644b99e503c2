"""The multi-rank path of bench.py on the CPU: every workload shards by independent units (noise
instances, shots, jobs), so ranks only meet at a barrier and a max-over-ranks of the timed region
(gloo, world size 2). A rank that fails makes the others' collective end with an error instead of
hanging (short process-group timeout)."""

from __future__ import annotations

import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return int(s.getsockname()[1])


def _rank(rank: int, world: int, port: int, value: float, fail: bool, out: mp.Queue) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))  # fmt: skip
    sys.path.insert(0, str(ROOT))
    import bench

    try:
        if fail:  # this rank leaves before joining
            out.put((rank, "left"))
            return
        d = bench.Dist(world, timeout_s=10)  # a missing peer ends the wait with an error
        d.barrier()
        out.put((rank, d.max(value)))
        d.close()
    except Exception as exc:  # noqa: BLE001 - reported to the test
        out.put((rank, f"error: {type(exc).__name__}"))


def _run(world: int, values: list[float], failing: set[int]) -> dict[int, object]:
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, values[r], r in failing, q)) for r in range(world)]
    for p in procs:
        p.start()
    results = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        if p.is_alive():
            p.kill()
    return results


def test_max_over_ranks_and_barrier():
    assert _run(2, [1.5, 4.0], set()) == {0: 4.0, 1: 4.0}


def test_a_rank_that_leaves_ends_the_others_collective():
    pytest.importorskip("torch")
    res = _run(2, [1.0, 2.0], {1})
    assert res[1] == "left"
    assert isinstance(res[0], str) and res[0].startswith("error")


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    d = bench.Dist(1)
    d.barrier()
    assert d.max(3.0) == 3.0
    d.close()
