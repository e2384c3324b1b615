"""The multi-GPU path of the bench on the CPU: two gloo ranks, each timing
its own replica windows; the job time is the slowest rank's, the job
throughput counts every rank's windows (weak scaling, no data-path
collective)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    r, w, _ = bench.dist_env()
    t = bench.max_over_ranks(times[rank], world, device="cpu")
    out.put((r, w, t, bench.job_throughput(t, world, nwin=51, steps=100)))
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_to_slowest():
    pytest.importorskip("torch.distributed")
    world, port = 2, _free_port()
    times = [800.0, 1000.0]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, times, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 for r in res)
    assert all(r[2] == 1000.0 for r in res)                      # the slowest rank
    assert all(abs(r[3] - 2 * 51 * 100 / 1.0) < 1e-9 for r in res)   # 10,200 window-steps/s


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.job_throughput(500.0, 1, 51, 100) == 51 * 100 / 0.5


def test_rebuild_cycle_amortisation_does_not_depend_on_the_step_count():
    """The bench's step is the step of qdyn's cycle, one list rebuild every
    25 steps, whatever --steps is: 20 timed steps (one rebuild) and 100 timed
    steps (four rebuilds) of the same per-step costs give the same figure."""
    import bench
    assert bench.first_rebuild_step(5) == 25 and bench.first_rebuild_step(25) == 25
    assert bench.first_rebuild_step(0) == 0 and bench.first_rebuild_step(26) == 50

    def run(steps, istep0):
        rb, pl = [], []
        for k in range(istep0, istep0 + steps):
            (rb if k % bench.NBCYCLE == 0 else pl).append(3.0 if k % bench.NBCYCLE == 0 else 0.5)
        return rb, pl
    a = bench.amortised_step_ms(*run(20, 25))
    b = bench.amortised_step_ms(*run(100, 25))
    assert a == b == (3.0 + 24 * 0.5) / 25
    assert bench.amortised_step_ms([2.0], []) == 2.0
    with pytest.raises(ValueError):
        bench.amortised_step_ms([], [1.0])
