"""Path-range sharding of one pricing request over ranks, and the merge of the shards' results.

The reference prices a request as one path range ``0..paths`` (crates/riga-engine/src/note.rs:
140-260, Sobol point ``n = path + 1``).  Paths are independent, so the range splits into
contiguous shards with no exchange while they run: rank ``r`` of ``world`` prices
``first_path = r * paths_per_rank`` and ``paths_per_rank`` paths, which are exactly paths
``r * paths_per_rank .. (r + 1) * paths_per_rank`` of the single-range run.  The one
collective is the gather of every shard's FP64 path sums (``rg_price_result.path_sums``,
16 doubles per scenario), merged on the root in rank order by ``rg_merge_results``; the merged
result equals the single-range result up to the order of the FP64 additions, and its event
counts are exact.
"""
from __future__ import annotations

import copy
import ctypes as C
from typing import List, Sequence

from . import abi


def shard_request(request, rank: int, world: int):
    """The request a rank prices: the same trade and market, its own contiguous path range.

    ``request.config.paths`` is the per-rank path count (weak scaling: the job prices
    ``world * paths`` paths).  The request's own ``first_path`` offsets the whole job.
    """
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} is outside a world of {world}")
    shard = copy.deepcopy(request)
    shard.options.first_path += rank * shard.config.paths
    return shard


def merge(lib, parts: Sequence[abi.PriceResult], total_paths: int) -> abi.PriceResult:
    """``rg_merge_results`` over the parts in the order given (rank order)."""
    n = len(parts)
    arr = (abi.PriceResult * n)()
    for i, p in enumerate(parts):
        C.memmove(C.byref(arr[i]), C.byref(p), C.sizeof(abi.PriceResult))
    out = abi.PriceResult()
    abi.check(lib, lib.rg_merge_results(arr, n, int(total_paths), C.byref(out)))
    return out


def gather_path_sums(results: Sequence[abi.PriceResult], group=None, device=None) -> List[List[List[float]]]:
    """All ranks' path sums, ``[rank][scenario][slot]``, through one ``all_gather``.

    Runs over whatever backend ``group`` uses (NCCL on GPUs, gloo on host cores); ``device``
    is where the gathered tensor lives (``cuda:<local rank>`` for NCCL, CPU for gloo).
    """
    import torch
    import torch.distributed as dist

    sums = torch.tensor([list(r.path_sums) for r in results], dtype=torch.float64, device=device)
    world = dist.get_world_size(group)
    gathered = [torch.empty_like(sums) for _ in range(world)]
    dist.all_gather(gathered, sums, group=group)
    return [g.cpu().tolist() for g in gathered]


def merge_gathered(lib, gathered: Sequence[Sequence[Sequence[float]]], paths_per_rank: int,
                   seed: int) -> List[abi.PriceResult]:
    """Per scenario, the merge of every rank's shard (``gathered`` as ``gather_path_sums`` returns)."""
    world = len(gathered)
    n_scen = len(gathered[0])
    merged = []
    for s in range(n_scen):
        parts = []
        for r in range(world):
            p = abi.PriceResult()
            p.path_sums[:] = list(gathered[r][s])
            p.seed = seed
            parts.append(p)
        merged.append(merge(lib, parts, paths_per_rank * world))
    return merged
