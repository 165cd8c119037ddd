"""Partition of independent problems and bands across ranks, and the host-side reductions
that follow the eigensolve (one process per GPU).

The CheFSI path itself has no data exchange between ranks: k-points and spins are independent
problems (DFT-FE's k-point pools), so a multi-GPU run gives each rank its own slice of them.
What crosses ranks are a few scalars per SCF step: the largest residual norm of the highest
occupied state over all k-points (the convergence test after the eigensolve) and the timing
maximum of a benchmark. These helpers take any torch.distributed process group (NCCL on GPUs,
gloo on CPU), or none for a single process.
"""
from __future__ import annotations

import numpy as np
import torch


def kpoint_pool_ranges(n_indices: int, n_pools: int) -> list[tuple[int, int]]:
    """[low, high) index range of every k-point pool, (-1, -1) for an empty pool.

    createKpointParallelizationIndices (utils/dftUtils.cc:244-274): pools take
    n_indices // n_pools + 1 consecutive indices each, the last non-empty one the remainder.
    Where that formula would run past n_indices (a middle pool holding the last, short
    block, e.g. 3 indices over 3 pools) the range is clipped to n_indices.
    """
    if n_pools < 1 or n_indices < 0:
        raise ValueError("need n_pools >= 1 and n_indices >= 0")
    per = n_indices // n_pools + 1
    out = []
    remaining = n_indices
    for i in range(n_pools):
        if remaining > 0:
            lo = i * per
            hi = lo + remaining if i == n_pools - 1 else (i + 1) * per
            out.append((lo, min(hi, n_indices)))
        else:
            out.append((-1, -1))
        remaining -= per
    return out


def band_group_ranges(n_bands: int, n_groups: int) -> list[tuple[int, int]]:
    """[low, high) band range of every band group (createBandParallelizationIndices,
    utils/dftUtils.cc:219-240): equal blocks of n_bands // n_groups, the last one extended to
    n_bands. Raises when a group would be empty, as the reference does."""
    if n_groups < 1:
        raise ValueError("need n_groups >= 1")
    size = n_bands // n_groups
    if size == 0:
        raise ValueError("more band groups than bands")
    out = [(i * size, (i + 1) * size) for i in range(n_groups)]
    out[-1] = (out[-1][0], n_bands)
    return out


def _reduce(x: float, op, group) -> float:
    import torch.distributed as dist
    if group is None and not (dist.is_available() and dist.is_initialized()):
        return float(x)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op, group=group)
    return float(t.item())


def max_over_ranks(x: float, group=None) -> float:
    """Maximum of a scalar over the ranks of group (the value itself without a group)."""
    import torch.distributed as dist
    return _reduce(x, dist.ReduceOp.MAX if dist.is_available() else None, group)


def sum_over_ranks(x: float, group=None) -> float:
    """Sum of a scalar over the ranks of group."""
    import torch.distributed as dist
    return _reduce(x, dist.ReduceOp.SUM if dist.is_available() else None, group)


def max_highest_occupied_residual(residual_norms_local, highest_state: int, group=None) -> float:
    """Largest residual norm of state highest_state over this rank's k-points, then over the
    pool group (computeMaximumHighestOccupiedStateResidualNorm,
    src/dft/kohnShamEigenSolve.cc:930-955). An empty pool contributes -1e6."""
    local = -1e6
    for r in residual_norms_local:
        local = max(local, float(np.asarray(r)[highest_state]))
    return max_over_ranks(local, group)
