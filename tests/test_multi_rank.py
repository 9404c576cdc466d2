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


def test_weak_scaling_shards_cover_the_finer_spectrum():
    """N ranks solve an N times finer spectrum, dealt round-robin: every energy
    exactly once, the same work per rank (within one energy)."""
    from fdmnes_gb300 import cluster as CL
    for world in (1, 2, 4, 8):
        all_e = CL.energy_grid(-5.0, 35.0, 0.1 / world)
        parts = [shard.energy_shard(len(all_e), r, world) for r in range(world)]
        assert sorted(sum(parts, [])) == list(range(len(all_e)))
        sizes = [len(p) for p in parts]
        assert max(sizes) - min(sizes) <= 1
        assert abs(max(sizes) - 401) <= 1


def _failing_worker(rank, world, port, out_dir):
    import datetime
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=5))
    if rank == 1:
        # a rank that fails between steps: it leaves without joining the gather
        dist.destroy_process_group()
        return
    outcome = "gathered"
    try:
        shard.gather_by_energy({0: 1.0}, 2)
    except Exception as exc:  # the collective times out or the peer is gone
        outcome = "failed: " + type(exc).__name__
    with open(os.path.join(out_dir, "r0.txt"), "w") as f:
        f.write(outcome)


def test_a_failed_rank_is_detected_on_the_host(tmp_path):
    """The surviving rank's gather ends with an error (5 s process-group
    timeout or the closed connection) instead of waiting forever."""
    port = _free_port()
    mp.spawn(_failing_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    assert (tmp_path / "r0.txt").read_text().startswith("failed")


def _fdm_worker(rank, world, port, energies, out_dir):
    """Rank `rank` solves its round-robin share of a small Cu spectrum (the
    oracle's FDM solve and Taull on the CPU, the per-rank work of the
    reference's energy loop) and gathers every energy's Taull."""
    import pickle
    import torch.distributed as dist
    import oracle
    from fdmnes_gb300 import abi, cluster as CL
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    st = CL.small_cu_structure()
    ga = abi.GridArgs(st)
    local = {}
    for k in shard.energy_shard(len(energies), rank, world):
        ei = CL.energy_inputs(st, energies[k])
        ri = CL.newind(st, ei.nlmsa, ei.nlmso)
        ea = abi.EnergyArgs(st, ei, ri)
        X, _ = oracle.mat_solve(ga, ea)
        local[k] = oracle.taull(ga, ea, X)
    res = shard.gather_by_energy(local, len(energies))
    with open(os.path.join(out_dir, f"fdm{rank}.pkl"), "wb") as f:
        pickle.dump(res, f)
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_fdm_spectrum_equals_single_process(tmp_path):
    """Two gloo ranks, each solving its round-robin share of a 5-energy FDM
    spectrum, gather the same Taull, bit for bit, as one process solving all
    energies."""
    import pickle
    import numpy as np
    import oracle
    from fdmnes_gb300 import abi, cluster as CL
    oracle.build()
    energies = [-5.0, 2.0, 9.0, 21.0, 35.0]
    port = _free_port()
    mp.spawn(_fdm_worker, args=(2, port, energies, str(tmp_path)), nprocs=2, join=True)
    r0 = pickle.load(open(tmp_path / "fdm0.pkl", "rb"))
    r1 = pickle.load(open(tmp_path / "fdm1.pkl", "rb"))
    st = CL.small_cu_structure()
    ga = abi.GridArgs(st)
    for k, E in enumerate(energies):
        ei = CL.energy_inputs(st, E)
        ri = CL.newind(st, ei.nlmsa, ei.nlmso)
        ea = abi.EnergyArgs(st, ei, ri)
        X, _ = oracle.mat_solve(ga, ea)
        T = oracle.taull(ga, ea, X)
        assert np.array_equal(r0[k], T) and np.array_equal(r1[k], T), E
