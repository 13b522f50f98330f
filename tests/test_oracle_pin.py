"""The oracle restatement against the reference's own code (CPU).

Golden vectors come from the reference's Basis / FourierTransform compiled
from its sources (tests/golden/make_golden.py).  The restatement must match
them bit for bit on x86 (same operation order); where oracle/_ref is present
the comparison is also made live on fresh inputs.
"""
import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as O

CASES = ["l12_e10", "l12_e10_g32", "l20_e10_g48", "l20_e10_g64", "l30_e25", "l40_e20"]


@pytest.mark.parametrize("name", CASES)
def test_basis_matches_reference_golden(name):
    g = load_golden(name)
    b = O.Basis(g["a"], float(g["ecut"]))
    assert b.ngw == int(g["ngw"]) and b.nrods == int(g["nrods"])
    assert tuple(b.np) == tuple(g["np"])
    assert tuple(b.idxmin) == tuple(g["idxmin"]) and tuple(b.idxmax) == tuple(g["idxmax"])
    for k in ("rod_h", "rod_k", "rod_lmin", "rod_size"):
        assert np.array_equal(getattr(b, k), g[k]), k
    sel = g["g_sel"]
    assert np.array_equal(b.kpg2[sel], g["kpg2_sel"])
    assert np.array_equal(b.kpgx.reshape(3, -1)[:, sel], g["kpgx_sel"])


def _weight_field(grid):
    n0, n1, n2 = grid
    k, j, i = np.meshgrid(np.arange(n2), np.arange(n1), np.arange(n0), indexing="ij")
    return (1.0 + 0.5 * np.cos(2 * np.pi * (i / n0 + 2 * j / n1 + 3 * k / n2))).reshape(-1)


@pytest.mark.parametrize("name", [c for c in CASES if not c.startswith(("l30", "l40"))])
def test_ft_matches_reference_golden(name):
    g = load_golden(name)
    b = O.Basis(g["a"], float(g["ecut"]))
    grid = tuple(int(x) for x in g["grid"])
    ft = O.FT(b, *grid)
    f1 = ft.backward(g["c1"])
    sel = g["f_sel"]
    # bit-identical where the platform rounds like the generator's (x86);
    # within a few ulps elsewhere
    np.testing.assert_allclose(f1[sel], g["f1_sel"], rtol=0, atol=1e-13 * np.abs(g["f1_sel"]).max())
    assert abs(np.vdot(f1, f1).real - float(g["f1_norm2"])) <= 1e-12 * float(g["f1_norm2"])
    r = ft.backward(g["c2"]) * _weight_field(grid)
    cr = ft.forward(r)
    np.testing.assert_allclose(cr, g["c_from_r"], rtol=0, atol=1e-13 * np.abs(g["c_from_r"]).max())
    rt = ft.forward(f1)
    np.testing.assert_allclose(rt, g["c1_roundtrip"], rtol=0, atol=1e-13 * np.abs(rt).max())
    if O.ref() is not None and np.dtype(np.float64).byteorder in "=<":
        import platform
        if platform.machine() in ("x86_64", "AMD64"):
            assert np.array_equal(f1[sel], g["f1_sel"])
            assert np.array_equal(cr, g["c_from_r"])


@pytest.mark.skipif(O.ref() is None, reason="reference not compiled here")
@pytest.mark.parametrize("L,ecut,grid", [(12.0, 10.0, (20, 24, 30)), (20.0, 10.0, (48, 48, 48)),
                                         (9.0, 7.5, (24, 20, 18))])
def test_ft_bit_identical_live(L, ecut, grid):
    a = np.diag([L, L, L]).reshape(9)
    b = O.Basis(a, ecut)
    rb = O.Basis(a, ecut, use_ref=True)
    for k in ("rod_h", "rod_k", "rod_lmin", "rod_size", "idx", "kpg2", "kpgx"):
        assert np.array_equal(getattr(b, k), getattr(rb, k))
    ft, rft = O.FT(b, *grid), O.RefFT(a, ecut, *grid)
    rng = np.random.default_rng(3)
    c = rng.standard_normal(b.ngw) + 1j * rng.standard_normal(b.ngw)
    assert np.array_equal(ft.backward(c), rft.backward(c))
    f = rng.standard_normal(ft.n012) + 1j * rng.standard_normal(ft.n012)
    assert np.array_equal(ft.forward(f), rft.forward(f))


def test_oracle_ft_matches_numpy():
    b = O.Basis(np.diag([12.0] * 3).reshape(9), 10.0)
    grid = (32, 32, 32)
    ft = O.FT(b, *grid)
    rng = np.random.default_rng(5)
    c = rng.standard_normal(b.ngw) + 1j * rng.standard_normal(b.ngw)
    F = np.zeros(grid[::-1], complex)
    idx = b.idx.reshape(-1, 3)
    F[idx[:, 2] % grid[2], idx[:, 1] % grid[1], idx[:, 0] % grid[0]] = c
    ref = np.fft.ifftn(F).ravel() * F.size
    got = ft.backward(c)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    assert np.abs(ft.forward(got) - c).max() <= 1e-13
