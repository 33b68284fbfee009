"""Multi-GPU partition of a search by code (PRN) range.

One process per GPU.  Every (job, code, Doppler) row of a search is
independent (FastSearchEngineBase runs its PRN loop as `par_unseq` with a
mutex only around the result vector, src/acquisition/fse.hpp:154, 273-294),
so rank r searches a contiguous range of each job's codes on its own device
and the per-code peak records are gathered on the host: a few dozen bytes per
code, the only exchange; there is no device-to-device collective.  The
gathered list, in code order, equals a single-device search of all codes.
"""
from __future__ import annotations

from typing import Callable, Sequence


def code_range(n_codes: int, rank: int, world: int) -> tuple[int, int]:
    """[start, stop) of the codes rank `rank` of `world` searches: contiguous,
    sizes differing by at most one, the larger ranges first."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of world {world}")
    if n_codes < 0:
        raise ValueError("negative code count")
    base, extra = divmod(n_codes, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def shard(items: Sequence, rank: int, world: int) -> list:
    """This rank's contiguous share of `items` (codes, code handles, ...)."""
    start, stop = code_range(len(items), rank, world)
    return list(items[start:stop])


def gather(local: list, world: int, group=None) -> list:
    """Concatenates every rank's `local` list in rank order (host objects over
    the process group: gloo on CPU, NCCL between GPUs)."""
    if world == 1:
        return list(local)
    import torch.distributed as dist
    parts: list = [None] * world
    dist.all_gather_object(parts, list(local), group=group)
    out: list = []
    for p in parts:
        out.extend(p)
    return out


def search(codes: Sequence, rank: int, world: int, search_codes: Callable[[list], list], group=None) -> list:
    """Runs `search_codes` (one device search over a list of codes, returning
    one peak record per code in order) on this rank's share and returns every
    code's record, in code order, on every rank."""
    return gather(search_codes(shard(codes, rank, world)), world, group)
