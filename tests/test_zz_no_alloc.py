"""qbg_backward_noalloc: the backward transform for callers that cannot
allocate device memory at call time (graph capture, pool-owned memory).

Called through the C ABI, twice in a row, and compared with qbg_backward on
the same input within the transform tolerance of the other tests (1e-13
relative).  Named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

import qball_gb300 as Q

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.mark.parametrize("L,ecut,grid,nb", [(12.0, 10.0, (32, 32, 32), 5),
                                            (20.0, 10.0, (48, 48, 48), 24),
                                            # 216-atom basis: one state per pass, three
                                            # passes reusing the static array
                                            (30.0, 25.0, (120, 120, 120), 3)])
def test_noalloc_backward_matches_backward_twice(cuda, L, ecut, grid, nb):
    import torch
    b = Q.Basis(L, ecut)
    ft = Q.FourierTransform(b, *grid)
    rng = np.random.default_rng(17)
    ld = b.ngw + 3
    c = np.zeros((nb, ld), complex)
    c[:, :b.ngw] = (rng.standard_normal((nb, b.ngw)) + 1j * rng.standard_normal((nb, b.ngw)))
    dc = torch.from_numpy(c).to(cuda)
    ref = torch.zeros((nb, ft.n012), dtype=torch.complex128, device=cuda)
    ft.backward(dc, ref, ldc=ld)
    L_ = Q.lib()
    for _ in range(2):
        out = torch.full((nb, ft.n012), 3.0 + 0j, dtype=torch.complex128, device=cuda)
        st = L_.qbg_backward_noalloc(ft.h, _p(dc), ld, _p(out), nb, None)
        assert st == 0, L_.qbg_last_error()
        torch.cuda.synchronize()
        assert _rel(out.cpu().numpy(), ref.cpu().numpy()) < 1e-13


def test_noalloc_rejects_oversized_grid(cuda):
    import torch
    b = Q.Basis(40.0, 20.0)
    ft = Q.FourierTransform(b, 160, 160, 160)
    c = torch.zeros((1, b.ngw), dtype=torch.complex128, device=cuda)
    f = torch.zeros((1, ft.n012), dtype=torch.complex128, device=cuda)
    st = Q.lib().qbg_backward_noalloc(ft.h, _p(c), b.ngw, _p(f), 1, None)
    assert st == 1
    assert b"static scratch" in Q.lib().qbg_last_error()
