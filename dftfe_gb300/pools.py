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


def world(group=None) -> tuple[int, int]:
    """(rank, size) in group, (0, 1) without an initialised process group."""
    import torch.distributed as dist
    if group is None and not (dist.is_available() and dist.is_initialized()):
        return 0, 1
    return dist.get_rank(group), dist.get_world_size(group)


def my_kpoints(n_k: int, group=None) -> range:
    """The k-point indices of this rank's pool (one pool per rank)."""
    rank, size = world(group)
    lo, hi = kpoint_pool_ranges(n_k, size)[rank]
    return range(lo, hi) if lo >= 0 else range(0)


def solve_kpoint_pool(n_k: int, solve_one, group=None) -> dict:
    """Run solve_one(k) for the k-points of this rank's pool only; {k: result}."""
    return {k: solve_one(k) for k in my_kpoints(n_k, group)}


def gather_over_pools(local: dict, n_k: int, n_states: int, group=None) -> np.ndarray:
    """[n_k, n_states] array of every pool's rows on every rank: this rank's rows in a
    zero-filled array, summed over the ranks (each row comes from exactly one pool), as the
    reference sums its per-pool k-point arrays over the inter-pool communicator."""
    import torch.distributed as dist
    out = np.zeros((n_k, n_states))
    for k, v in local.items():
        out[k] = np.asarray(v, dtype=np.float64)[:n_states]
    rank, size = world(group)
    if size == 1:
        return out
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.from_numpy(out).to(dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()


C_KB = 3.166811429e-06   # Boltzmann constant in Ha / K


def _fermi_dirac_sums(x: float, eig_local, weights_local, T: float, spin_factor: float):
    """Local sums of the occupation count and of its derivative at Fermi level x over this
    rank's k-points (FermiDiracFunctionValue / FermiDiracFunctionDerivativeValue,
    src/dft/fermiEnergy.cc:26-97: the logistic function evaluated on the side where its
    exponential does not overflow)."""
    f = d = 0.0
    kT = C_KB * T
    for ev, w in zip(eig_local, weights_local):
        t1 = (np.asarray(ev, dtype=np.float64) - x) / kT
        neg = t1 <= 0.0
        e = np.exp(np.where(neg, t1, -t1))
        t2 = 1.0 / (1.0 + e)
        occ = np.where(neg, t2, e * t2)
        f += spin_factor * w * occ.sum()
        d += spin_factor * w * (e / kT * t2 * t2).sum()
    return f, d


def fermi_energy(eig_local, weights_local, n_electrons: float, T: float,
                 spin_polarized: bool = False, group=None) -> float:
    """Fermi energy over all k-point pools (dftClass::compute_fermienergy,
    src/dft/fermiEnergy.cc:102-230, the k-point build): bisection on [min, max] of all pools'
    eigenvalues until the electron-count residual is at most 1e-9 (100 steps at most), then
    Newton-Raphson to 1e-10; every step sums the pools' local counts over the ranks. eig_local /
    weights_local: this rank's k-points' eigenvalues and weights."""
    import torch.distributed as dist
    sf = 1.0 if spin_polarized else 2.0
    lo_local = min((float(np.min(e)) for e in eig_local), default=np.inf)
    hi_local = max((float(np.max(e)) for e in eig_local), default=-np.inf)
    x_r = max_over_ranks(hi_local, group)
    x_l = -max_over_ranks(-lo_local, group)

    def count(x):
        f, _ = _fermi_dirac_sums(x, eig_local, weights_local, T, sf)
        return sum_over_ranks(f, group) - n_electrons

    y_r, y_l = count(x_r), count(x_l)
    if y_l * y_r > 0.0:
        raise RuntimeError("Fermi energy: bisection bracket has no sign change")
    fe, R = x_l, abs(y_l)
    for it in range(100):
        xb = 0.5 * (x_l + x_r)
        yb = count(xb)
        if yb * y_l > 0.0:
            x_l = xb
        else:
            x_r = xb
        if abs(yb) <= 1e-9 or it == 99:
            fe, R = xb, abs(yb)
            break
    it = 0
    while R > 1e-10 and it < 100:
        f, d = _fermi_dirac_sums(fe, eig_local, weights_local, T, sf)
        f, d = sum_over_ranks(f, group), sum_over_ranks(d, group)
        r = f - n_electrons
        R = abs(r)
        fe -= r / d
        it += 1
    if R > 1e-10:
        raise RuntimeError("Fermi energy: Newton-Raphson did not converge")
    return fe


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
