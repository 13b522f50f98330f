"""The in-place, in-order 120-point prime-factor transform of the whole-plane
and z-pass kernels, restated on the CPU: the same Ruritanian map
n = (15 n1 + 40 a + 24 b) mod 120 indexes input and output, so the transform
is a 3-point DFT over a (direction s), a 5-point and an 8-point DFT with the
opposite root.  Checks the slot sets the kernels use (PlPass<0..2> in
qbg_pfa.cuh: item bases and strides) against numpy's FFT in both
directions, and that every pass touches each of the 120 slots exactly once.
"""
import numpy as np
import pytest


def _base(p, j):
    """PlPass<p>::base(j), the slot step and the radix of the pass."""
    if p == 0:  # j = 5 n1 + b, 3-point over a
        n1, b = divmod(j, 5)
        return (15 * n1 + 24 * b) % 120, 40, 3
    if p == 1:  # j = 3 n1 + a, 5-point over b
        n1, a = divmod(j, 3)
        return (15 * n1 + 40 * a) % 120, 24, 5
    a, b = divmod(j, 5)  # j = 5 a + b, 8-point over n1
    return (40 * a + 24 * b) % 120, 15, 8


def _slots(p, j):
    base, step, r = _base(p, j)
    return [(base + step * k) % 120 for k in range(r)]


def _dft(v, s):
    n = len(v)
    k = np.arange(n)
    return np.exp(s * 2j * np.pi * np.outer(k, k) / n) @ v


def _transform(x, s, order=(0, 1, 2)):
    x = x.astype(complex).copy()
    signs = {0: s, 1: -s, 2: -s}  # 3-point with s, 5- and 8-point opposite
    for p in order:
        nitems = {0: 40, 1: 24, 2: 15}[p]
        for j in range(nitems):
            sl = _slots(p, j)
            x[sl] = _dft(x[sl], signs[p])
    return x


@pytest.mark.parametrize("p,nitems", [(0, 40), (1, 24), (2, 15)])
def test_each_pass_partitions_the_slots(p, nitems):
    seen = sorted(i for j in range(nitems) for i in _slots(p, j))
    assert seen == list(range(120))


@pytest.mark.parametrize("order", [(0, 1, 2), (2, 1, 0), (1, 0, 2)])
def test_in_place_in_order_transform_is_the_dft(order):
    rng = np.random.default_rng(4)
    x = rng.standard_normal(120) + 1j * rng.standard_normal(120)
    bwd = _transform(x, +1, order)  # y_k = sum_j x_j exp(+2 pi i jk/n)
    fwd = _transform(x, -1, order)
    assert np.abs(bwd - 120 * np.fft.ifft(x)).max() < 1e-12 * np.abs(x).sum()
    assert np.abs(fwd - np.fft.fft(x)).max() < 1e-12 * np.abs(x).sum()


def test_fused_eight_point_items_around_a_pointwise_product():
    """The backward 8-point pass, a pointwise product and the forward
    8-point pass touch the same slots item by item, so one register-resident
    item can run all three (the v(r) product of k_plane_vloc)."""
    rng = np.random.default_rng(5)
    x = rng.standard_normal(120) + 1j * rng.standard_normal(120)
    v = rng.standard_normal(120)
    ref = np.fft.fft(v * (120 * np.fft.ifft(x)))
    y = _transform(x, +1, (0, 1))
    for j in range(15):
        sl = _slots(2, j)
        u = _dft(y[sl], -1)           # backward 8-point (opposite root)
        u = u * v[sl]                 # v at the output positions: in order
        y[sl] = _dft(u, +1)           # forward 8-point
    y = _transform(y, -1, (1, 0))
    assert np.abs(y - ref).max() < 1e-11 * np.abs(ref).max()
