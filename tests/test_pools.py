"""Host-side multi-rank logic: k-point pool and band-group partitions (the reference's
formulas) and the scalar reductions that follow the eigensolve, over a world_size-2 gloo
process group on CPU."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from dftfe_gb300 import pools


@pytest.mark.parametrize("n,P,expect", [
    (8, 2, [(0, 5), (5, 8)]),
    (4, 3, [(0, 2), (2, 4), (-1, -1)]),
    (5, 3, [(0, 2), (2, 4), (4, 5)]),
    (3, 3, [(0, 2), (2, 3), (-1, -1)]),
    (1, 4, [(0, 1), (-1, -1), (-1, -1), (-1, -1)]),
    (7, 1, [(0, 7)]),
])
def test_kpoint_pool_ranges(n, P, expect):
    got = pools.kpoint_pool_ranges(n, P)
    assert got == expect
    covered = [i for lo, hi in got if lo >= 0 for i in range(lo, hi)]
    assert covered == list(range(n))


def test_band_group_ranges():
    assert pools.band_group_ranges(10, 3) == [(0, 3), (3, 6), (6, 10)]
    assert pools.band_group_ranges(8, 1) == [(0, 8)]
    with pytest.raises(ValueError):
        pools.band_group_ranges(2, 3)


def test_single_process_reductions_are_identity():
    assert pools.max_over_ranks(2.5) == 2.5
    assert pools.sum_over_ranks(-1.0) == -1.0
    assert pools.max_highest_occupied_residual([np.array([0.1, 0.3]), np.array([0.2, 0.05])], 1) == 0.3


def test_single_process_pool_helpers():
    """Without a process group: one pool holds every k-point, the gathered array is the local
    one, and the Fermi level puts the requested electron count into the states (spin-degenerate
    and spin-polarised counting, src/dft/fermiEnergy.cc:26-60), between the highest fully and
    the lowest empty level at low temperature."""
    assert list(pools.my_kpoints(5)) == [0, 1, 2, 3, 4]
    solved = pools.solve_kpoint_pool(3, lambda k: np.arange(4.0) + k)
    assert sorted(solved) == [0, 1, 2]
    ev = pools.gather_over_pools(solved, 3, 4)
    assert np.array_equal(ev, np.arange(4.0)[None, :] + np.arange(3.0)[:, None])
    eig = [np.array([-1.0, -0.5, 0.3, 0.8])] * 2
    w = [0.5, 0.5]
    for spin_polarized, ne in ((False, 4.0), (True, 2.0)):
        fe = pools.fermi_energy(eig, w, ne, 300.0, spin_polarized=spin_polarized)
        f, _ = pools._fermi_dirac_sums(fe, eig, w, 300.0, 1.0 if spin_polarized else 2.0)
        assert abs(f - ne) < 1e-9
        assert -0.5 < fe < 0.3


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n_k, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        lo, hi = pools.kpoint_pool_ranges(n_k, world)[rank]
        mine = range(lo, hi) if lo >= 0 else range(0)
        # residual norms of the highest occupied state: k-point k has 0.01 * (k + 1)
        res = [np.array([0.0, 0.01 * (k + 1)]) for k in mine]
        r = pools.max_highest_occupied_residual(res, 1)
        s = pools.sum_over_ranks(float(len(mine)))
        t = pools.max_over_ranks(10.0 + rank)
        out.put((rank, r, s, t))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("n_k", [5, 1])
def test_pool_reductions_over_two_gloo_ranks(n_k):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n_k, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, r, s, t in res:
        assert abs(r - 0.01 * n_k) < 1e-15     # the last k-point's residual, on every rank
        assert s == n_k                        # every k-point counted once
        assert t == 11.0


def test_partitions_cover_every_index_once():
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies

    @hyp.given(st.integers(0, 500), st.integers(1, 64))
    @hyp.settings(max_examples=300, deadline=None)
    def kpoints(n, P):
        got = pools.kpoint_pool_ranges(n, P)
        assert len(got) == P
        covered = [i for lo, hi in got if lo >= 0 for i in range(lo, hi)]
        assert covered == list(range(n))
        # non-empty pools come first, each a contiguous block of at most n // P + 1
        sizes = [hi - lo for lo, hi in got if lo >= 0]
        assert all(0 < s <= n // P + 1 for s in sizes)

    @hyp.given(st.integers(1, 500), st.integers(1, 64))
    @hyp.settings(max_examples=300, deadline=None)
    def bands(n, G):
        if n // G == 0:
            with pytest.raises(ValueError):
                pools.band_group_ranges(n, G)
            return
        got = pools.band_group_ranges(n, G)
        assert [i for lo, hi in got for i in range(lo, hi)] == list(range(n))

    kpoints()
    bands()


N_STATES, N_ELECTRONS, T_FERMI = 8, 8.0, 500.0


def _bloch_eigenvalues(k):
    """Lowest N_STATES eigenvalues of Hamiltonian k of the 32-entry Bloch set (degree-2 cells
    so that the CPU test stays fast; the oracle's dense Hermitian operator)."""
    from dftfe_gb300 import problems
    from tests.helpers import dense_operator
    pr = problems.bloch_set(32, p=2, small=True)[k]
    return np.linalg.eigvalsh(dense_operator(pr))[:N_STATES]


def _pool_worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        solved = pools.solve_kpoint_pool(32, _bloch_eigenvalues)
        ev = pools.gather_over_pools(solved, 32, N_STATES)
        mine = [solved[k] for k in sorted(solved)]
        fe = pools.fermi_energy(mine, [1.0 / 32] * len(mine), N_ELECTRONS, T_FERMI)
        out.put((rank, sorted(solved), ev, fe))
    finally:
        dist.destroy_process_group()


def test_bloch_set_over_two_kpoint_pools():
    """The 32 Bloch Hamiltonians split over two k-point pools (ranks of a gloo group): each
    rank solves only its pool's range (kpoint_pool_ranges: 0..16 and 17..31), every rank then
    holds all 32 eigenvalue rows (summed over the pools) and the same Fermi energy, and both
    equal the single-process results."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_pool_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ranges = pools.kpoint_pool_ranges(32, 2)
    assert [r[1] for r in res] == [list(range(*ranges[0])), list(range(*ranges[1]))]
    ref = np.array([_bloch_eigenvalues(k) for k in range(32)])
    fe_ref = pools.fermi_energy(list(ref), [1.0 / 32] * 32, N_ELECTRONS, T_FERMI)
    for _, _, ev, fe in res:
        assert np.abs(ev - ref).max() < 1e-12
        assert abs(fe - fe_ref) < 1e-12
    # the electron count at the Fermi energy
    f, _ = pools._fermi_dirac_sums(fe_ref, list(ref), [1.0 / 32] * 32, T_FERMI, 2.0)
    assert abs(f - N_ELECTRONS) < 1e-9
