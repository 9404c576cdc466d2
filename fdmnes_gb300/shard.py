"""Energy sharding across GPU processes (one process per GPU).

The reference distributes the energies of a spectrum round-robin over its MPI
ranks: rank r of P computes energy ie = ie0 + (je - 1) * P + r
(source/fdm.f90:3484-3497), then rank 0 gathers every energy's Taull
(MPI_RECV_Tau, source/fdm.f90:4623-4664).  Energies are independent, so the
device path has no collective: each process solves its own energies in one
batch and the host gathers the small per-energy results.
"""
from __future__ import annotations

from typing import Dict, List, Sequence


def energy_shard(n_energies: int, rank: int, world: int) -> List[int]:
    """0-based energy indices of ``rank`` under the reference's round-robin rule."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return list(range(rank, n_energies, world))


def gather_by_energy(local: Dict[int, object], n_energies: int, group=None) -> List[object]:
    """All-gather {energy index: result} dicts over torch.distributed and return
    the results in energy order.  Every index must come from exactly one rank."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    parts: List[Dict[int, object]] = [None] * world  # type: ignore[list-item]
    dist.all_gather_object(parts, local, group=group)
    out: List[object] = [None] * n_energies
    seen = set()
    for p in parts:
        for k, v in p.items():
            if k in seen:
                raise RuntimeError(f"energy {k} computed twice")
            seen.add(k)
            out[k] = v
    missing = [k for k in range(n_energies) if k not in seen]
    if missing:
        raise RuntimeError(f"energies never computed: {missing[:8]}")
    return out


def balanced_shard(costs: Sequence[float], rank: int, world: int) -> List[int]:
    """Cost-balanced alternative: greedy longest-processing-time assignment."""
    order = sorted(range(len(costs)), key=lambda k: -costs[k])
    load = [0.0] * world
    owner = [0] * len(costs)
    for k in order:
        r = min(range(world), key=lambda q: load[q])
        owner[k] = r
        load[r] += costs[k]
    return sorted(k for k in range(len(costs)) if owner[k] == rank)
