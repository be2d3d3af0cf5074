"""The N > 1 layout on CPU: two gloo ranks shard the cosmology sample with no
data-path collective and agree on the job's step time (max over ranks)."""
import os
import socket

import pytest
import torch.multiprocessing as tmp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    from discoeb_gb300.sharding import dist_env, max_over_ranks, shard
    from discoeb_gb300.workloads import sample_cosmologies

    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, _ = dist_env()
    params, _ = sample_cosmologies(3 * w, seed=5)
    mine = [params[i] for i in shard(3, w, r)]
    t = max_over_ranks(1.0 + r)
    out.put((r, [p["Omegam"] for p in mine], t))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_shard_and_reduce_the_step_time():
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    from discoeb_gb300.workloads import sample_cosmologies

    full, _ = sample_cosmologies(6, seed=5)
    assert res[0][1] + res[1][1] == [p["Omegam"] for p in full]   # disjoint, complete, in order
    assert res[0][2] == res[1][2] == 2.0                           # max over ranks


def test_shard_rejects_bad_ranks():
    from discoeb_gb300.sharding import shard

    assert list(shard(2, 3, 1)) == [2, 3]
    with pytest.raises(ValueError):
        shard(2, 2, 2)
