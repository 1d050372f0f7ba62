"""The N > 1 bench path on CPU: two gloo ranks (replicas of the workload, no
data-path collective).  Checks the whole-job aggregation (units of all ranks
over the slowest rank's time), the barrier, and that only rank 0 reports."""
import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, q) -> None:
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    r, w, lr = bench.dist_env()
    dist = bench.dist_init(w)
    bench.barrier(dist)
    # rank r processed (r + 1) * 1e6 units in (1 + r) seconds
    value, tmax = bench.aggregate((r + 1) * 1e6, 1.0 + r, dist)
    bench.barrier(dist)
    q.put((r, w, lr, value, tmax))
    dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_over_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[:3] for o in out] == [(0, 2, 0), (1, 2, 1)]
    for _, _, _, value, tmax in out:
        assert tmax == 2.0
        assert value == 3e6 / 2.0


def test_reference_arm_runs_on_rank_0_only():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.run_reference(None, bench.WORKLOADS["c1"], rank=1) is None


def test_single_process_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.dist_init(1) is None
    assert bench.aggregate(5e6, 2.0, None) == (2.5e6, 2.0)
