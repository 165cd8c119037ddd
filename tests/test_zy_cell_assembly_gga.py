"""Real GGA cell Hamiltonians on the device (chefsi_assemble_cell_hamiltonians_gga), their Bloch
form, and the cell Hamiltonians of cells of any shape (chefsi_assemble_cell_hamiltonians_geometry)
against the oracle's q-loops. Tolerance 1e-12 relative (FP64 sums in another order). Collected
after the other GPU files and before the allocation-free entry point's file.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.helpers import small_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def C(cuda):
    from dftfe_gb300 import chefsi
    return chefsi


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("p", [2, 4])
def test_gga_cell_assembly_matches_oracle(C, p):
    """On-device real GGA cell matrices against the oracle's q-loop (p = 4: ragged tiles)."""
    from tests.helpers import shape_tables
    pr = small_problem(n=2, L=4.0, p=p, wells=2)
    mesh = pr.mesh
    N, dN, w3 = shape_tables(mesh)
    vjxw = pr.info["vjxw"]
    g = np.random.default_rng(p).standard_normal((mesh.n_cells, len(w3), 3)) * w3[None, :, None]
    K_ = mesh.stiffness_cell()
    ref = orc.cell_hamiltonians_gga_direct(K_, N, dN, vjxw, g)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()
    out = C.assemble_cell_hamiltonians_gga(t(N), t(dN), t(K_), t(vjxw), t(g)).cpu().numpy()
    assert rel(out, ref) < 1e-12


@pytest.mark.parametrize("p", [2, 4])
def test_bloch_gga_cell_assembly_matches_oracle(C, p):
    """On-device Bloch GGA cell matrices for two k-points against the oracle's q-loop, and the
    GGA-free launch of the same entry family unchanged."""
    from tests.helpers import shape_tables
    K = [0.2, -0.1, 0.3]
    pr = small_problem(n=2, L=4.0, p=p, wells=2, kpoint=K)
    mesh = pr.mesh
    N, dN, w3 = shape_tables(mesh)
    jxw = np.broadcast_to(w3, (mesh.n_cells, len(w3))).copy()
    vjxw = pr.info["vjxw"]
    g = np.random.default_rng(p + 10).standard_normal((mesh.n_cells, len(w3), 3)) * w3[None, :, None]
    kp = np.array([K, [0.5, 0.25, -0.4]])
    K_ = mesh.stiffness_cell()
    ref = orc.cell_hamiltonians_bloch_direct(K_, N, dN, vjxw, jxw, kp, g)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()
    out = C.assemble_cell_hamiltonians_bloch(t(N), t(dN), t(K_), t(vjxw), t(jxw), kp,
                                             gga_jxw=t(g)).cpu().numpy()
    assert rel(out, ref) < 1e-12
    lda = C.assemble_cell_hamiltonians_bloch(t(N), t(dN), t(K_), t(vjxw), t(jxw), kp[:1])
    assert rel(lda.cpu().numpy()[0], pr.cell_mats) < 1e-12


@pytest.mark.parametrize("p", [2, 4])
def test_geometry_cell_assembly_matches_oracle(C, p):
    """Cells of any shape: a different Jacobian factor at every quadrature point of every cell
    (random symmetric positive definite, scaled like J^-1 J^-T JxW of the mesh) against the
    oracle's q-loop; with the uniform mesh's factors the result is the workload's own cell
    matrices (0.5 K + N^T diag(v) N)."""
    from tests.helpers import shape_tables
    pr = small_problem(n=2, L=4.0, p=p, wells=2)
    mesh = pr.mesh
    N, dN, w3 = shape_tables(mesh)
    h = mesh.h
    dNref = dN * h
    vjxw = pr.info["vjxw"]
    nq = len(w3)
    rng = np.random.default_rng(20 + p)
    R = rng.standard_normal((mesh.n_cells, nq, 3, 3)) * 0.3 + np.eye(3)
    F = np.einsum('cqik,cqjk->cqij', R, R) * (w3 / h ** 2)[None, :, None, None]
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()
    out = C.assemble_cell_hamiltonians_geometry(t(N), t(dNref), t(F), t(vjxw)).cpu().numpy()
    ref = orc.cell_hamiltonians_geometry_direct(N, dNref, F, vjxw)
    assert rel(out, ref) < 1e-12
    Fu = np.broadcast_to(np.eye(3)[None, None] * (w3 / h ** 2)[None, :, None, None],
                         (mesh.n_cells, nq, 3, 3))
    out = C.assemble_cell_hamiltonians_geometry(t(N), t(dNref), t(Fu), t(vjxw)).cpu().numpy()
    assert rel(out, pr.cell_mats) < 1e-12
