"""bench.py --gpus N runs N independent realisations (one per rank, no
collective on the data path); the host logic around them is checked here
with two gloo ranks on the CPU: distinct seeds, max-over-ranks timings and the
whole-job throughput that rank 0 prints."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = [0.2 + 0.1 * rank, 0.3 - 0.1 * rank]  # this rank's step and e2e times
    step, e2e = bench.max_over_ranks(t, dist, "cpu")
    val = bench.job_cells_per_s(64 ** 3, world, step)
    out.put((rank, bench.rank_seed(4001, rank), step, e2e, val))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_gloo():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, s0, st0, e0, v0), (r1, s1, st1, e1, v1) = res
    assert s0 != s1
    assert abs(st0 - 0.3) < 1e-12 and abs(st1 - 0.3) < 1e-12
    assert abs(e0 - 0.3) < 1e-12 and abs(e1 - 0.3) < 1e-12
    assert abs(v0 - 2 * 64 ** 3 / 0.3) < 1e-6 * v0 and v0 == v1
