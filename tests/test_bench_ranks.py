"""bench.py's whole-job figures over ranks, on CPU with two gloo ranks: the timed region is
the slowest rank's and the walk steps are the sum over ranks (weak scaling: each rank solves
its own copy of the workload with its own seeds)."""
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2")
    import torch.distributed as tdist
    tdist.init_process_group("gloo", rank=rank, world_size=2)
    sys.path.insert(0, ROOT)
    import bench
    seconds, steps = bench.reduce_over_ranks(1.5 + rank, 1000 * (rank + 1), True, "cpu")
    out.put((rank, seconds, steps))
    tdist.barrier()
    tdist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time_and_the_sum_of_steps():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(out.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert got == [(0, 2.5, 3000.0), (1, 2.5, 3000.0)]


def test_one_rank_keeps_its_own_figures():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_over_ranks(1.25, 77, False, "cpu") == (1.25, 77)
