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


def _species_fixture():
    g = load_golden("species_xe_ar")
    return g, [dict(tau=g[f"tau{i}"], twnl=g[f"twnl{i}"], lproj=g[f"lproj{i}"], wt=g[f"wt{i}"])
               for i in range(len(g["names"]))]


def test_species_tables_fixture_shapes_and_symmetry():
    """The testsuite species tables: KB projector count per species (nlm of
    Species: nchannels * sum_{l != llocal} (2l+1)), l order of
    NonLocalPotential::init, l = 1 and 2 rows that are the real harmonics times
    one radial function, and the radial projectors' values at |G| = 0 (zero
    for l > 0)."""
    g, sp = _species_fixture()
    for i, s in enumerate(sp):
        info = g[f"info{i}"]
        lmax, lloc, nch, nlm = (int(x) for x in info[:4])
        assert len(s["lproj"]) == nlm == s["twnl"].shape[0]
        assert s["twnl"].shape[1] == int(O.Basis(g["a"], float(g["ecut"])).ngw)
        expect = [l for l in range(lmax + 1) if l != lloc for _ in range(nch)
                  for _ in range(2 * l + 1)]
        assert list(s["lproj"]) == expect
        vn = g[f"vnlg{i}"]
        for l in range(1, lmax + 1):
            if l != lloc:
                assert np.all(vn[l, :, 0] == 0.0)
        # the three l = 1 rows of a channel square-sum to (3/4pi) v^2
        r = [k for k, l in enumerate(s["lproj"]) if l == 1][:3]
        if r:
            tw = s["twnl"][r]
            ss = (tw * tw).sum(0)
            A = g["A"]
            kq = O.Basis(g["a"], float(g["ecut"])).kpgx.reshape(3, -1) - A[:, None]
            gmag = np.sqrt((kq * kq).sum(0))
            lch = [k for k, l in enumerate(s["lproj"]) if l == 1].index(r[0]) // 3
            v = np.interp(gmag, g[f"vnlg_g{i}"], vn[1, lch])
            mask = (gmag > 0.5) & (gmag < 3.0)
            assert np.allclose(ss[mask], 3.0 / (4 * np.pi) * v[mask] ** 2, rtol=2e-2)


def test_oracle_table_path_equals_synthetic_path():
    """The oracle's caller-table path of NonLocalPotential::energy, fed the
    tables its synthetic path builds, gives the synthetic path's H|psi> and
    E_nl bit for bit."""
    import qball_gb300 as Q
    from qball_gb300 import synth
    cell = synth.make_cell("t12")
    b = O.Basis(Q.cubic_cell(cell.L), cell.ecut)
    ft = O.FT(b, *cell.grid)
    v = synth.vlocal(cell)
    sp = synth.species(cell)
    A = synth.kick()
    h1 = O.Ham(ft, v, sp)
    h1.set_A(A)
    na, npr = len(sp[0]["tau"]), (cell.lmax + 1) ** 2
    rows = [h1.projector(ipr * na) for ipr in range(npr)]
    sp2 = [dict(tau=sp[0]["tau"], twnl=np.array([r[0] for r in rows]),
                lproj=np.array([r[1] for r in rows]), wt=np.array([r[2] for r in rows]))]
    h2 = O.Ham(ft, v, sp2)
    h2.set_A(A)
    rng = np.random.default_rng(1)
    c = rng.standard_normal((b.ngw, 3)) + 1j * rng.standard_normal((b.ngw, 3))
    occ = np.full(3, 2.0)
    r1, e1 = h1.hpsi(c, occ)
    r2, e2 = h2.hpsi(c, occ)
    assert np.array_equal(r1, r2) and e1 == e2


@pytest.mark.skipif(O.ref() is None, reason="reference checker not built here")
def test_species_tables_fixture_matches_reference_species():
    """Live pin: the fixture's radial projectors and KB weights are those of
    the reference's own Species (read and initialised now from the testsuite
    files)."""
    import os
    root = os.environ.get("QBG_REFERENCE", "")
    g, sp = _species_fixture()
    path0 = os.path.join(root, "testsuite", "pseudopotentials", str(g["files"][0]))
    if not root or not os.path.exists(path0):
        pytest.skip("reference tree not available")
    for i in range(len(sp)):
        h = O.ref_species_load(os.path.join(root, "testsuite", "pseudopotentials",
                                            str(g["files"][i])), 1.0)
        info = O.ref_species_info(h)
        assert np.array_equal(info, g[f"info{i}"])
        gg = g[f"vnlg_g{i}"]
        for l in range(info[0] + 1):
            for ic in range(info[2]):
                assert np.array_equal(O.ref_species_vnlg(h, l, ic, gg), g[f"vnlg{i}"][l, ic])
        O.ref_species_destroy(h)
