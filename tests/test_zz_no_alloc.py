"""The allocation-free Cholesky step against the allocating driver.

gx_cholesky_step_noalloc serves callers that cannot let a library allocate
device memory (they own all of it through their own pool or a hard cap, and
cannot afford the device-wide synchronisation of cudaMalloc/cudaFree).  It
must reproduce, step for step, the factor rows and the next pivot that the
allocating entry point gx_cholesky produces.  This file is collected last so
that a failure here never hides another test.
"""

import ctypes

import numpy as np
import pytest

import giaoint_gb300 as gi
from giaoint_gb300 import _native as nat
from giaoint_gb300.cholesky import _cholesky_columns, _cholesky_diagonal

pytestmark = pytest.mark.gpu
ATOL = 1e-12


def two_shell_basis():
    return gi.Basis([gi.Shell((0.2, -0.1, 0.3), 2, [0.8], [1.0]), gi.Shell((-0.3, 0.4, -0.2), 3, [0.6], [1.0])])


@pytest.mark.parametrize("B", [(0.05, -0.03, 0.2), (0.0, 0.0, 0.0)])
def test_noalloc_step_matches_allocating_driver(B):
    torch = pytest.importorskip("torch")
    basis = two_shell_basis()
    field = gi.MagneticField(B, (0.37, -0.29, 0.43))
    real = all(x == 0 for x in B)
    ref = gi.cholesky_eri(basis, field=field, threshold=1e-8)
    assert len(ref.pivots) > 3
    n = basis.ao_count
    N = n * n
    ns = len(basis.shells)
    diag = _cholesky_diagonal(basis, [(a, b) for a in range(ns) for b in range(a, ns)], field=field)
    dev = torch.device("cuda:0")
    vdtype = torch.float64 if real else torch.complex128
    residual = torch.tensor(diag.ravel(), dtype=torch.float64, device=dev)
    factors = torch.zeros((2, N), dtype=vdtype, device=dev)
    result = torch.zeros(3, dtype=torch.float64, device=dev)  # gx_cholesky_step_result (24 bytes)
    lib = nat.lib()
    for k in range(2):  # two calls in a row; the second reads the first's output row
        mu, nu = (int(x) for x in ref.pivots[k])
        pivot = mu * n + nu
        column = _cholesky_columns(basis, [(mu, nu)], field=field)[0]
        col = torch.from_numpy(np.ascontiguousarray(column)).to(dev)
        rc = lib.gx_cholesky_step_noalloc(ctypes.c_void_p(factors.data_ptr()), k, pivot,
                                          ctypes.c_void_p(col.data_ptr()), n, int(real),
                                          ctypes.c_void_p(residual.data_ptr()),
                                          ctypes.c_void_p(factors[k].data_ptr()),
                                          ctypes.c_void_p(result.data_ptr()), None)
        nat.check(rc)
        torch.cuda.synchronize()
        row = factors[k].cpu().numpy()
        expected = ref.vectors[k].ravel()
        assert np.abs(row - (expected.real if real else expected)).max() <= ATOL
        raw = result.cpu().numpy()
        max_res = float(raw[0])
        argmax = int(raw[1:2].view(np.int64)[0])
        res_host = residual.cpu().numpy()
        assert max_res == pytest.approx(res_host.max(), abs=1e-15)
        nxt = int(ref.pivots[k + 1][0]) * n + int(ref.pivots[k + 1][1])
        # the next pivot agrees unless the residual gap is a tie (<= 1e-10)
        assert argmax == nxt or abs(res_host[argmax] - res_host[nxt]) <= 1e-10
        assert float(raw[2]) >= -1e-12


def test_noalloc_rejects_oversized_and_bad_arguments():
    lib = nat.lib()
    rc = lib.gx_cholesky_step_noalloc(None, 0, 0, ctypes.c_void_p(16), 257, 1, ctypes.c_void_p(16),
                                      ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert rc == -3 and "n <= 256" in nat.last_error()
    rc = lib.gx_cholesky_step_noalloc(None, 0, 5 * 5, ctypes.c_void_p(16), 5, 1, ctypes.c_void_p(16),
                                      ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert rc == -2
    rc = lib.gx_cholesky_step_noalloc(None, 1, 0, ctypes.c_void_p(16), 5, 1, ctypes.c_void_p(16),
                                      ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert rc == -1
