"""bench.py's multi-rank logic on CPU: two gloo ranks (world size 2) take the
contract's barrier, the maximum of the timed spans and the sum of the
particle-steps over ranks; the reference arm prints on rank 0 only; the
replicas use different seeds."""
import io
import multiprocessing as mp
import os
import socket
import sys
from contextlib import redirect_stdout
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), GPAT_DIST_BACKEND="gloo")
    sys.path[:0] = [str(REPO), str(REPO / "stochastic-parker_gb300")]
    import bench
    import torch.distributed as dist
    world, r, local = bench.dist_setup()
    bench.barrier(world)
    span = bench.max_over_ranks(world, 1.5 + r, "cpu")
    total = bench.sum_over_ranks(world, 10.0 * (r + 1), "cpu")
    out = io.StringIO()
    if r == 1:
        args = bench.parse_args(["--impl", "reference"])
        with redirect_stdout(out):
            bench.run_reference(args, world, r)
    bench.barrier(world)
    dist.destroy_process_group()
    q.put((r, world, span, total, out.getvalue()))


def test_two_gloo_ranks_reduce_like_the_contract():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=240) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, world, span, total, printed in res:
        assert world == 2 and span == 2.5 and total == 30.0
        assert printed == ""          # rank 1 of the reference arm prints nothing


def test_replicas_have_distinct_seeds():
    pytest.importorskip("torch")
    sys.path[:0] = [str(REPO)]
    import bench
    args = bench.parse_args(["--grid", "64", "--scale", "1e-4"])
    seeds = {bench.make_workload(args, 1, seed=2 + r, nframes=1).params["seed"] for r in range(2)}
    assert len(seeds) == 2


def test_headline_extras_record_a_failure(monkeypatch):
    """The headline line's extra configurations: each is measured by its own
    workload function, a failing one is recorded with its error, and the
    others (and the headline) are kept."""
    sys.path[:0] = [str(REPO), str(REPO / "stochastic-parker_gb300")]
    import bench
    seen = []

    def fake_ours(a, world, rank, local):
        seen.append((a.workload, a.steps, a.warmup, a.no_accuracy))
        return {"value": 1.0, "unit": "particle-steps/s", "config": {"workload": a.workload},
                "not_kept": 0}

    def fake_batch(a, world, rank, local):
        raise RuntimeError("out of memory")

    def fake_learned(a, world, rank, local):
        seen.append((a.workload, a.scale))
        return {"value": 2.0, "unit": "particle-steps/s", "ms_per_step": 1.0, "config": {},
                "clocks": {}, "learned_splitting": {"arms": {}}}

    monkeypatch.setattr(bench, "run_ours", fake_ours)
    monkeypatch.setattr(bench, "run_batch", fake_batch)
    monkeypatch.setattr(bench, "run_learned", fake_learned)
    args = bench.parse_args([])
    out = bench.other_configs(args, 0)
    assert out["turbulence_3d_256"] == {"value": 1.0, "unit": "particle-steps/s",
                                        "config": {"workload": "turbulence_3d"}}
    assert out["batched_shock_2d_64"] == {"error": "RuntimeError: out of memory"}
    assert out["learned_3d_scale_0.1"]["value"] == 2.0
    assert ("turbulence_3d", 1, 1, True) in seen and ("learned_3d", 0.1) in seen
