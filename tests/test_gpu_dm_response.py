"""First-order density-matrix response (densityMatrixEigenBasisFirstOrderResponse) through the
C ABI against the FP64 oracle.

H' is the difference of two seeded Kohn-Sham cell-matrix sets on the same mesh (a potential
perturbation: the kinetic parts cancel). Tolerances: FP64 X P' 1e-10 relative and
densityMatDerFermiEnergy 1e-12 relative; mixed (tensor-core H X, Gram, rotation) 2e-5.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.helpers import dense_operator, small_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def chefsi(cuda):
    from dftfe_gb300 import chefsi as C
    return C


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def setup(C, n=3, L=6.0, p=2, N=24):
    pr = small_problem(n=n, L=L, p=p, projectors=True)
    pr2 = small_problem(n=n, L=L, p=p, seed=5, wells=3)
    pert = pr2.cell_mats - pr.cell_mats
    op_prime = C.KohnShamOperator(pr.cell_map, pert, pr.sqrt_mass, pr.inv_sqrt_mass, pr.n_dofs)
    ora_prime = orc.OracleOperator(pr.cell_map, pert, pr.inv_sqrt_mass, pr.n_dofs)
    w, Q = np.linalg.eigh(dense_operator(pr))
    return op_prime, ora_prime, Q[:, :N].copy(), w[:N].copy()


@pytest.mark.parametrize("T", [500.0, 5000.0, 50000.0])
def test_dm_response_fp64_matches_oracle(chefsi, T):
    op_prime, ora_prime, X, eig = setup(chefsi)
    mu = 0.5 * (eig[10] + eig[11])
    XP_o, dmu_o = orc.density_matrix_first_order_response(ora_prime, X, eig, mu, T)
    Xt = torch.from_numpy(X.copy()).cuda()
    dmu = chefsi.densityMatrixEigenBasisFirstOrderResponse(op_prime, Xt, eig, mu, T)
    assert rel(Xt.cpu().numpy(), XP_o) < 1e-10
    assert rel(dmu, dmu_o) < 1e-12


def test_dm_response_mixed_close_to_oracle(chefsi):
    # N = 128 on 1728 dofs puts the H X, Gram and rotation on the tensor cores
    op_prime, ora_prime, X, eig = setup(chefsi, n=4, L=8.0, p=3, N=128)
    mu = 0.5 * (eig[60] + eig[61])
    XP_o, dmu_o = orc.density_matrix_first_order_response(ora_prime, X, eig, mu, 3000.0)
    Xt = torch.from_numpy(X.copy()).cuda()
    dmu = chefsi.densityMatrixEigenBasisFirstOrderResponse(op_prime, Xt, eig, mu, 3000.0,
                                                          precision="mixed")
    assert rel(Xt.cpu().numpy(), XP_o) < 2e-5
    assert rel(dmu, dmu_o) < 1e-12


def test_dm_response_rejects_bad_arguments(chefsi):
    from dftfe_gb300._lib import ChefsiError
    op_prime, _, X, eig = setup(chefsi)
    Xt = torch.from_numpy(X.copy()).cuda()
    with pytest.raises(ValueError):
        chefsi.densityMatrixEigenBasisFirstOrderResponse(op_prime, Xt, eig[:-1], 0.0, 500.0)
    with pytest.raises(ChefsiError):
        chefsi.densityMatrixEigenBasisFirstOrderResponse(op_prime, Xt, eig, 0.0, 0.0)
