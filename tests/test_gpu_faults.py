"""Failure detection on the GPU path, made on the host (no GPU fault): injected allocation
failure, a non-SPD overlap handed to the Cholesky, non-finite operator input. Each must come
back as a status code with the context still usable."""
import numpy as np
import pytest
import torch

from tests.helpers import small_problem

pytestmark = pytest.mark.gpu


@pytest.fixture()
def C(cuda):
    from dftfe_gb300 import chefsi
    return chefsi


def test_not_spd_overlap_is_reported(C, monkeypatch):
    from dftfe_gb300 import _lib
    pr = small_problem(projectors=True)
    op = C.KohnShamOperator.from_problem(pr)
    X = torch.from_numpy(pr.initial_vectors()).cuda()
    monkeypatch.setenv("CHEFSI_FAULT_INJECT", "not_spd")
    with pytest.raises(_lib.ChefsiError) as ei:
        C.pseudoGramSchmidtOrthogonalization(op, X)
    assert ei.value.code == _lib.CHEFSI_ERR_NOT_SPD
    monkeypatch.delenv("CHEFSI_FAULT_INJECT")
    C.pseudoGramSchmidtOrthogonalization(op, X)       # context still usable
    Y = X.cpu().numpy()
    assert np.abs(Y.T @ Y - np.eye(Y.shape[1])).max() < 1e-12


def test_rank_deficient_overlap_is_not_spd(C):
    from dftfe_gb300 import _lib
    pr = small_problem(projectors=True)
    op = C.KohnShamOperator.from_problem(pr)
    X = torch.zeros((pr.n_dofs, 6), dtype=torch.float64, device="cuda")
    with pytest.raises(_lib.ChefsiError) as ei:
        C.pseudoGramSchmidtOrthogonalization(op, X)
    assert ei.value.code == _lib.CHEFSI_ERR_NOT_SPD


def test_nan_input_is_rejected(C):
    from dftfe_gb300 import _lib
    pr = small_problem()
    pr.cell_mats[0, 0, 0] = np.nan
    with pytest.raises(_lib.ChefsiError) as ei:
        C.KohnShamOperator.from_problem(pr)
    assert ei.value.code == _lib.CHEFSI_ERR_NAN


def test_alloc_failure_is_reported(C, monkeypatch):
    from dftfe_gb300 import _lib
    pr = small_problem()
    monkeypatch.setenv("CHEFSI_FAULT_INJECT", "alloc")
    with pytest.raises(_lib.ChefsiError) as ei:
        C.KohnShamOperator.from_problem(pr)
    assert ei.value.code == _lib.CHEFSI_ERR_ALLOC
    monkeypatch.delenv("CHEFSI_FAULT_INJECT")
    op = C.KohnShamOperator.from_problem(pr)           # recovers
    assert op.n_dofs == pr.n_dofs


def test_bad_map_is_rejected(C):
    from dftfe_gb300 import _lib
    pr = small_problem()
    pr.cell_map[0, 0] = pr.n_dofs + 5
    with pytest.raises(_lib.ChefsiError) as ei:
        C.KohnShamOperator.from_problem(pr)
    assert ei.value.code == _lib.CHEFSI_ERR_INVALID
