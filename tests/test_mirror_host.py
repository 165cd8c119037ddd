"""Host logic of the Python mirror on CPU, against a fake of the C library (no GPU): the
spectrum-split dispatch of solve() and the Loewdin scaling around the solver's
densityMatrixEigenBasisFirstOrderResponse."""
import ctypes

import numpy as np
import pytest
import torch

from dftfe_gb300 import chefsi


def _arr(ptr, n):
    return np.ctypeslib.as_array((ctypes.c_double * n).from_address(ptr.value))


class FakeLib:
    def __init__(self, n_dofs):
        self.M = n_dofs
        self.calls = []

    def chefsi_solver_create(self, p, h):
        return 0

    def chefsi_solver_destroy(self, h):
        return 0

    def chefsi_solve_spectrum_split(self, h, op, X, N, n_occ, XF, eig, res, cr, first, st):
        nfr = N - n_occ
        self.calls.append(("ss", N, n_occ, XF.value))
        _arr(eig, nfr)[:] = np.arange(nfr) + 0.5
        _arr(res, nfr)[:] = 1e-3
        return 0

    def chefsi_density_matrix_first_order_response(self, op, X, ld, N, eig, mu, T, dmu, prec, st):
        x = _arr(X, self.M * N)
        self.calls.append(("dm", x.copy(), mu, T, prec))
        x *= 3.0
        _arr(dmu, N)[:] = 1.0
        return 0


class FakeOp:
    handle = ctypes.c_void_p(0)

    def __init__(self, M):
        self.sq = torch.linspace(0.5, 2.0, M, dtype=torch.float64)

    def getSqrtMassVec(self):
        return self.sq

    def getInvSqrtMassVec(self):
        return 1.0 / self.sq


@pytest.fixture
def fake(monkeypatch):
    M = 7
    lib = FakeLib(M)
    monkeypatch.setattr(chefsi._lib, "load", lambda *a, **k: lib)
    monkeypatch.setattr(chefsi, "_stream", lambda stream=None: ctypes.c_void_p(0))
    return lib, FakeOp(M), M


def test_solve_with_fewer_eigenvalues_takes_the_spectrum_split(fake):
    lib, op, M = fake
    s = chefsi.ChebyshevOrthogonalizedSubspaceIterationSolver()
    X = torch.zeros((M, 5), dtype=torch.float64)
    XF = torch.zeros((M, 2), dtype=torch.float64)
    ev, rn = np.zeros(2), np.zeros(5)
    out_ev, out_rn = s.solve(op, X, ev, rn, eigenVectorsRotFracDensity=XF)
    assert lib.calls[0][:3] == ("ss", 5, 3) and lib.calls[0][3] == XF.data_ptr()
    assert out_ev is ev and np.allclose(ev, [0.5, 1.5])
    assert np.allclose(rn[:2], 1e-3)
    with pytest.raises(ValueError):
        s.solve(op, X, np.zeros(2), None)


def test_solver_response_scales_into_and_out_of_the_loewdin_basis(fake):
    lib, op, M = fake
    s = chefsi.ChebyshevOrthogonalizedSubspaceIterationSolver()
    X0 = torch.from_numpy(np.random.default_rng(0).standard_normal((M, 3)))
    X = X0.clone()
    dmu = s.densityMatrixEigenBasisFirstOrderResponse(op, X, np.array([0.1, 0.2, 0.3]), 0.15,
                                                      500.0)
    _, seen, mu, T, prec = lib.calls[0]
    assert np.allclose(seen.reshape(M, 3), (X0 * op.sq[:, None]).numpy(), rtol=1e-15)
    assert (mu, T, prec) == (0.15, 500.0, chefsi._lib.PREC_FP64)
    assert torch.allclose(X, 3.0 * X0, rtol=1e-14)
    assert np.all(dmu == 1.0)
