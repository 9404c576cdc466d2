"""Energy sharding over CPU ranks (gloo, world size 2): the host logic of the
multi-GPU path, which has no device collective."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from fdmnes_gb300 import shard


def test_round_robin_rule():
    # source/fdm.f90:3484-3497: ie = ie0 + (je-1)*P + rank
    parts = [shard.energy_shard(10, r, 3) for r in range(3)]
    assert parts == [[0, 3, 6, 9], [1, 4, 7], [2, 5, 8]]
    assert sorted(sum(parts, [])) == list(range(10))
    with pytest.raises(ValueError):
        shard.energy_shard(4, 2, 2)


def test_balanced_shard_covers_all():
    costs = [5, 1, 1, 1, 4, 2, 2, 3]
    parts = [shard.balanced_shard(costs, r, 2) for r in range(2)]
    assert sorted(parts[0] + parts[1]) == list(range(len(costs)))
    loads = [sum(costs[k] for k in p) for p in parts]
    assert abs(loads[0] - loads[1]) <= max(costs)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard.energy_shard(n, rank, world)
    local = {k: (k * k, rank) for k in mine}
    res = shard.gather_by_energy(local, n)
    with open(os.path.join(out_dir, f"r{rank}.txt"), "w") as f:
        f.write(repr(res))
    dist.barrier()
    dist.destroy_process_group()


def test_gather_over_two_gloo_ranks(tmp_path):
    port = _free_port()
    mp.spawn(_worker, args=(2, port, 7, str(tmp_path)), nprocs=2, join=True)
    r0 = eval(open(tmp_path / "r0.txt").read())
    r1 = eval(open(tmp_path / "r1.txt").read())
    assert r0 == r1
    assert [v[0] for v in r0] == [k * k for k in range(7)]
    assert [v[1] for v in r0] == [k % 2 for k in range(7)]
