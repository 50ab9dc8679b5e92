"""The N > 1 path of bench.py on CPU: two gloo ranks shard the k-point
batches of the band path (no data collective) and reduce the timer by max,
through fame.shard, the helpers bench.py uses.  No GPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import fame.shard as S


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, steps, nb, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, _ = S.env_rank()
    mine = S.batches_of(r, w, steps, nb)
    t_local = 1.0 + 0.5 * r                    # a slower rank 1
    t_max = S.max_over_ranks(t_local)
    dist.barrier()
    q.put((r, mine, t_max))
    dist.destroy_process_group()


@pytest.mark.parametrize("steps,nb", [(5, 5), (3, 5), (4, 2)])
def test_two_gloo_ranks_shard_and_reduce(steps, nb):
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, steps, nb, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    # each step round gives the ranks distinct batches while there are enough
    for s in range(steps):
        got = [o[1][s] for o in out]
        if nb >= world:
            assert len(set(got)) == world
        assert got == [(s * world + r) % nb for r in range(world)]
    # every rank sees the slowest rank's time
    assert all(abs(o[2] - 1.5) < 1e-12 for o in out)
    assert S.whole_job_rate(8, steps, world, 1.5) == pytest.approx(8 * steps * world / 1.5)


def test_single_process_defaults():
    assert S.max_over_ranks(2.5) == 2.5
    assert S.batches_of(0, 1, 3, 5) == [0, 1, 2]
