"""The allocation-free eigensolver entry point (chefsi_syevd_noalloc) against chefsi_syevd.

chefsi_syevd_noalloc serves callers that cannot allocate device memory while they solve
(their pool allocator owns the GPU's memory, or they cannot take cudaFree's device-wide
synchronisation). It keeps its workspace in one file-scope device array, so it is limited
to N <= 256. This test calls both entry points through the C ABI (ctypes on
libchefsi_gb300.so) on two matrices in a row -- the second call finds the first call's
leftovers in the shared array -- and requires the same eigenvalues (1e-12 relative) and the
same eigenvectors up to sign (1e-10); after a warm-up call, a call must leave the device's free
memory unchanged. This file is collected after every other test file on purpose.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _sym(n, seed, degenerate=False):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    w = np.sort(rng.standard_normal(n))
    if degenerate:
        w[5:9] = w[5]
    A = (Q * w) @ Q.T
    return 0.5 * (A + A.T)


def _call(fn, A):
    n = A.shape[0]
    a = torch.from_numpy(A).cuda().contiguous()
    w = torch.empty(n, dtype=torch.float64, device="cuda")
    Z = torch.empty((n, n), dtype=torch.float64, device="cuda")
    rc = fn(n, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(w.data_ptr()),
            ctypes.c_void_p(Z.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return rc, w.cpu().numpy(), Z.cpu().numpy()


def test_syevd_noalloc_matches_syevd(cuda):
    from dftfe_gb300 import _lib
    lib = _lib.load()
    for i, (n, degenerate) in enumerate([(200, False), (256, True)]):
        A = _sym(n, 100 + i, degenerate)
        rc0, w0, Z0 = _call(lib.chefsi_syevd, A)
        rc1, w1, Z1 = _call(lib.chefsi_syevd_noalloc, A)
        assert rc0 == 0 and rc1 == 0, lib.chefsi_last_error()
        assert np.abs(w1 - w0).max() <= 1e-12 * max(1.0, np.abs(w0).max())
        # eigenvectors equal up to sign inside each eigenvalue's (possibly degenerate) space
        P0 = Z0 @ np.diag(np.sign(np.sum(Z0, 0) + 1e-300))
        P1 = Z1 @ np.diag(np.sign(np.sum(Z1, 0) + 1e-300))
        sep = np.abs(np.diff(w0)) > 1e-8
        ok = np.concatenate([[True], sep]) & np.concatenate([sep, [True]])
        assert np.abs(P1[:, ok] - P0[:, ok]).max() < 1e-10
        assert np.abs(Z1.T @ Z1 - np.eye(n)).max() < 1e-10
        assert np.abs(A @ Z1 - Z1 * w1).max() < 1e-10 * max(1.0, np.abs(w1).max())


def test_syevd_noalloc_allocates_nothing_after_warmup(cuda):
    """After one warm-up call on the device (which places the array in device memory: the
    runtime loads device code lazily), a call leaves the device's free memory unchanged; the
    operands are created before the measurement."""
    from dftfe_gb300 import _lib
    lib = _lib.load()
    n = 128
    A = _sym(n, 3)
    _call(lib.chefsi_syevd_noalloc, A)  # warm-up
    a = torch.from_numpy(A).cuda().contiguous()
    w = torch.empty(n, dtype=torch.float64, device="cuda")
    Z = torch.empty((n, n), dtype=torch.float64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    rc = lib.chefsi_syevd_noalloc(n, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(w.data_ptr()),
                                  ctypes.c_void_p(Z.data_ptr()), stream)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert rc == 0, lib.chefsi_last_error()
    assert free1 == free0


def test_syevd_noalloc_rejects_oversize(cuda):
    from dftfe_gb300 import _lib
    lib = _lib.load()
    A = _sym(257, 7)
    rc, _, _ = _call(lib.chefsi_syevd_noalloc, A)
    assert rc == _lib.CHEFSI_ERR_INVALID
    assert b"257" in lib.chefsi_last_error()
