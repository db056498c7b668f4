"""bench.py with --gpus N > 1, on the host: every rank runs an independent replica of the solve (it
does not shard), and the timed region is bracketed by a barrier over the ranks and reported as the
slowest rank's time.  Two gloo ranks on 127.0.0.1 check that plumbing (rank and world from the
launcher's environment, the barrier, the max over ranks) without a GPU."""
import importlib.util
import os
import socket

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    spec = importlib.util.spec_from_file_location("bench_replica", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    r, local, w, pg = bench.dist_setup(world)
    bench.barrier(pg)
    slowest = bench.max_over_ranks(pg, 10.0 + 5.0 * r)   # rank r's "time": the slowest counts
    bench.barrier(pg)
    q.put((r, local, w, slowest))
    pg.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 0, 2, 15.0), (1, 1, 2, 15.0)]


def test_one_rank_needs_no_process_group():
    spec = importlib.util.spec_from_file_location("bench_single", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK") if k in os.environ}
    try:
        r, local, w, pg = bench.dist_setup(1)
    finally:
        os.environ.update(env)
    assert (r, local, w, pg) == (0, 0, 1, None)
    assert bench.max_over_ranks(pg, 3.5) == 3.5
