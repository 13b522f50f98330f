"""Parity of the sm_103a path (through the C ABI) against the CPU oracle.

Tolerances: the plain FP64 form must match the oracle to <= 1e-10 relative
(H|psi>, rho(r), the current and psi after N ETRS steps); the transforms to
<= 1e-12.  The mixed form (FP32 transforms and projector GEMMs, FP64
Taylor accumulation) is held to 5e-5 relative on psi after 3 steps.
"""
import numpy as np
import pytest

from conftest import rel_err
import qball_gb300 as Q
from qball_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NT = 8  # oracle threads


def _torch():
    import torch
    return torch


def setup(name, prec="fp64", **kw):
    cell = synth.make_cell(name, **kw)
    b = Q.Basis(cell.L, cell.ecut)
    H = Q.Hamiltonian(b, *cell.grid, precision=prec)
    v = synth.vlocal(cell)
    H.set_vlocal(v)
    H.set_nonlocal(synth.species(cell))
    ob = O.Basis(b.a, cell.ecut)
    oft = O.FT(ob, *cell.grid)
    oh = O.Ham(oft, v, synth.species(cell))
    psi = synth.wavefunctions(cell, b)
    return cell, b, H, oft, oh, psi


def dev(x):
    torch = _torch()
    return torch.from_numpy(np.ascontiguousarray(x)).to("cuda:0")


@pytest.mark.parametrize("name", ["l12_e10", "l12_e10_g32", "l20_e10_g48", "l20_e10_g64"])
def test_fft_backward_forward_vs_reference_golden(cuda, name):
    from conftest import load_golden
    g = load_golden(name)
    b = Q.Basis(g["a"], float(g["ecut"]))
    grid = tuple(int(x) for x in g["grid"])
    ft = Q.FourierTransform(b, *grid)
    torch = _torch()
    c = dev(np.stack([g["c1"], g["c2"]]))
    f = torch.zeros((2, ft.n012), dtype=torch.complex128, device=cuda)
    ft.backward(c, f)
    fh = f.cpu().numpy()
    sel = g["f_sel"]
    assert rel_err(fh[0][sel], g["f1_sel"]) < 1e-13
    assert abs(np.vdot(fh[0], fh[0]).real / float(g["f1_norm2"]) - 1) < 1e-13
    # forward of w(r) * backward(c2): the rs_mul_add shape
    n0, n1, n2 = grid
    k, j, i = np.meshgrid(np.arange(n2), np.arange(n1), np.arange(n0), indexing="ij")
    w = (1.0 + 0.5 * np.cos(2 * np.pi * (i / n0 + 2 * j / n1 + 3 * k / n2))).reshape(-1)
    r = dev(np.stack([fh[0], fh[1] * w]))
    out = torch.zeros((2, b.ngw), dtype=torch.complex128, device=cuda)
    ft.forward(r, out)
    oh = out.cpu().numpy()
    assert rel_err(oh[0], g["c1_roundtrip"]) < 1e-13
    assert rel_err(oh[1], g["c_from_r"]) < 1e-13


@pytest.mark.parametrize("L,ecut,grid", [(12.0, 10.0, (32, 32, 32)), (12.0, 10.0, (20, 24, 30)),
                                         (20.0, 10.0, (48, 48, 48)), (10.0, 6.0, (28, 28, 28)),
                                         (10.0, 6.0, (22, 22, 26)),
                                         (12.0, 10.0, (120, 48, 40)),
                                         (12.0, 10.0, (120, 120, 40)),
                                         (12.0, 10.0, (72, 80, 144)),
                                         (12.0, 10.0, (160, 36, 50))])
def test_fft_vs_oracle_many_grids(cuda, L, ecut, grid):
    """radix 2,3,4,5,8, the direct-DFT primes 7, 11 and 13, and the
    prime-factor lengths 120 = 8x15, 48 = 16x3, 40 = 8x5, 72 = 8x9,
    80 = 16x5, 144 = 16x9, and 160 (the 512-atom cell's length, Stockham);
    120 x 120 planes run through the whole-plane kernels"""
    b = Q.Basis(L, ecut)
    ob = O.Basis(b.a, ecut)
    oft = O.FT(ob, *grid)
    ft = Q.FourierTransform(b, *grid)
    rng = np.random.default_rng(11)
    nb = 3
    c = rng.standard_normal((nb, b.ngw)) + 1j * rng.standard_normal((nb, b.ngw))
    torch = _torch()
    f = torch.zeros((nb, ft.n012), dtype=torch.complex128, device=cuda)
    ft.backward(dev(c), f)
    fh = f.cpu().numpy()
    for s in range(nb):
        assert rel_err(fh[s], oft.backward(c[s])) < 1e-13
    r = rng.standard_normal((nb, ft.n012)) + 1j * rng.standard_normal((nb, ft.n012))
    out = torch.zeros((nb, b.ngw), dtype=torch.complex128, device=cuda)
    ft.forward(dev(r), out)
    oh = out.cpu().numpy()
    for s in range(nb):
        assert rel_err(oh[s], oft.forward(r[s])) < 1e-13


def test_fft_padded_leading_dimension(cuda):
    b = Q.Basis(12.0, 10.0)
    ft = Q.FourierTransform(b, 32, 32, 32)
    ld = b.ngw + 37
    rng = np.random.default_rng(2)
    c = np.zeros((4, ld), complex)
    c[:, :b.ngw] = rng.standard_normal((4, b.ngw)) + 1j * rng.standard_normal((4, b.ngw))
    torch = _torch()
    f = torch.zeros((4, ft.n012), dtype=torch.complex128, device=cuda)
    ft.backward(dev(c), f, ldc=ld)
    out = torch.full((4, ld), 7.0 + 0j, dtype=torch.complex128, device=cuda)
    ft.forward(f, out, ldc=ld)
    oh = out.cpu().numpy()
    assert np.abs(oh[:, :b.ngw] - c[:, :b.ngw]).max() < 1e-13
    assert np.all(oh[:, b.ngw:] == 7.0)  # padding rows untouched


@pytest.mark.parametrize("name,gemm", [("t12", "ozaki"), ("c1", "ozaki"), ("c1", "simt")])
def test_hpsi_fp64_vs_oracle(cuda, name, gemm):
    cell, b, H, oft, oh, psi = setup(name)
    H.set_fp64_gemm(gemm)
    occ = synth.occupations(cell)
    torch = _torch()
    out = torch.zeros_like(dev(psi))
    enl = H.hpsi(dev(psi), out, occ, want_enl=True)
    ref, enl_ref = oh.hpsi(psi.T, occ, nthreads=NT)
    assert rel_err(out.cpu().numpy(), ref.T) < 1e-10
    assert abs(enl - enl_ref) <= 1e-10 * abs(enl_ref)
    # Hermiticity <phi|H psi> = <H phi|psi>
    hp = out.cpu().numpy()
    m = psi.conj() @ hp.T
    assert np.abs(m - m.conj().T).max() < 1e-10 * np.abs(m).max()


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("mixed_df32", 2e-6)])
def test_hpsi_216_atom_grid(cuda, prec, tol):
    """The 120^3 grid and 161 235-wave basis of the 216-atom cell (register
    lane-group y pass, 15 x 8), with 8 atoms and 4 states to keep the oracle
    quick."""
    cell, b, H, oft, oh, psi = setup("c2", prec=prec, natoms=8, nst=4)
    occ = synth.occupations(cell)
    torch = _torch()
    out = torch.zeros_like(dev(psi))
    H.hpsi(dev(psi), out, occ)
    ref, _ = oh.hpsi(psi.T, occ, nthreads=NT)
    assert rel_err(out.cpu().numpy(), ref.T) < tol


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("mixed_df32", 2e-6)])
def test_hpsi_216_atom_grid_full_chunk(cuda, prec, tol):
    """The 216-atom cell's 120^3 grid and basis with 40 states: one full
    32-state transform chunk plus a last chunk of 8, the tensor-core GEMM1
    split over K, and E_nl."""
    cell, b, H, oft, oh, psi = setup("c2", prec=prec, natoms=8, nst=40)
    H.set_chunk(32)
    occ = synth.occupations(cell)
    torch = _torch()
    out = torch.zeros_like(dev(psi))
    enl = H.hpsi(dev(psi), out, occ, want_enl=True)
    ref, enl_ref = oh.hpsi(psi.T, occ, nthreads=NT)
    assert rel_err(out.cpu().numpy(), ref.T) < tol
    assert abs(enl - enl_ref) <= tol * abs(enl_ref)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("mixed_df32", 1e-11)])
def test_density_216_atom_grid(cuda, prec, tol):
    """The density on the 216-atom cell's 120^3 grid (the whole-plane kernel:
    x and y transforms of a plane and w |psi(r)|^2 in one CTA) against the
    oracle, 40 states: a full 32-state chunk and an accumulating chunk of 8."""
    cell, b, H, oft, oh, psi = setup("c2", prec=prec, natoms=8, nst=40)
    H.set_chunk(32)
    occ = synth.occupations(cell)
    torch = _torch()
    rho = torch.zeros(oft.n012, dtype=torch.float64, device=cuda)
    nel = H.update_density(dev(psi), occ, rho)
    rref, nref = O.update_density(oft, psi.T, occ, nthreads=NT)
    assert rel_err(rho.cpu().numpy(), rref) < tol
    assert abs(nel - nref) < tol * nref


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-13), ("mixed_df32", 1e-12)])
@pytest.mark.parametrize("ecut", [25.0, 35.0])
def test_plane_kernel_matches_band_row_kernels(cuda, prec, tol, ecut):
    """On 120 x 120 planes the whole-plane kernel (fused 2), the band-row
    fused kernel (1) and the separate x, y, x kernels (0) give the same
    H|psi> and density to the rounding of the transform arithmetic.  At the
    216-atom cell's cutoff the Z row of a plane (3577 rods) is staged in the
    plane's 52 non-band rows; at the higher cutoff (5005 rods, 40 non-band
    rows) it does not fit and the plane fills straight from HBM."""
    cell, b, H, oft, oh, psi = setup("c2", prec=prec, natoms=8, nst=6, ecut=ecut)
    occ = synth.occupations(cell)
    torch = _torch()
    p = dev(psi)
    outs, rhos = [], []
    for fused in (2, 1, 0):
        H.set_transform_config(0, 1, fused, 1)
        assert H.transform_config()["fused"] == fused
        out = torch.zeros_like(p)
        H.hpsi(p, out, occ)
        rho = torch.zeros(oft.n012, dtype=torch.float64, device=cuda)
        H.update_density(p, occ, rho)
        outs.append(out.cpu().numpy())
        rhos.append(rho.cpu().numpy())
    for k in (1, 2):
        assert rel_err(outs[k], outs[0]) < tol, k
        assert rel_err(rhos[k], rhos[0]) < tol, k


@pytest.mark.parametrize("name", ["c1", "c1q"])
def test_etrs_and_density_c1_grids_vs_oracle(cuda, name):
    """One ETRS step and the density of the 8-atom cell on the 48^3 grid and
    on the reference's own dense-grid rule for it (64^3), FP64, against the
    oracle: psi(t+dt), the density of the predicted state built inside
    update(), its electron count, and the density of psi(t+dt)."""
    cell, b, H, oft, oh, psi = setup(name)
    occ = synth.occupations(cell)
    A = synth.kick()
    torch = _torch()
    p = dev(psi)
    rho = torch.zeros(oft.n012, dtype=torch.float64, device=cuda)
    nel = H.etrs_step(p, occ, 0.05, A_t=A, A_tdt=A, rho=rho, want_nel=True)
    oh.set_A(A)
    ref, rref, nref = oh.etrs_step(psi.T.copy(), occ, 0.05, A, A, want_rho=True, nthreads=NT)
    assert rel_err(p.cpu().numpy(), ref.T) < 1e-10
    assert rel_err(rho.cpu().numpy(), rref) < 1e-10
    assert abs(nel - nref) < 1e-10 * nref
    rho2 = torch.zeros_like(rho)
    nel2 = H.update_density(p, occ, rho2)
    rref2, nref2 = O.update_density(oft, ref, occ)
    assert rel_err(rho2.cpu().numpy(), rref2) < 1e-10
    assert abs(nel2 - nref2) < 1e-10 * nref2


@pytest.mark.parametrize("name,kw,slices,tol", [("c1", {}, 7, 1e-13), ("c1", {}, 6, 1e-11),
                                                ("t12b", {}, 7, 1e-13),
                                                ("c2", dict(natoms=8, nst=40), 7, 1e-13)])
def test_fp64_tensor_core_gemm_matches_fp64_fma_gemm(cuda, name, kw, slices, tol):
    """The plain form's projector GEMMs on the tensor cores (Ozaki scheme:
    7-bit integer slices, exact FP32 windows) against the same form's FP64
    FMA GEMMs on the same inputs: H|psi> and E_nl agree to the rounding of
    the slices (49 bits for 7 slices, 42 for 6)."""
    cell, b, H, oft, oh, psi = setup(name, **kw)
    occ = synth.occupations(cell)
    torch = _torch()
    p = dev(psi)
    outs, enls = {}, {}
    for mode in ("simt", "ozaki"):
        H.set_fp64_gemm(mode, slices)
        o = torch.zeros_like(p)
        enls[mode] = H.hpsi(p, o, occ, want_enl=True)
        outs[mode] = o.cpu().numpy()
    assert rel_err(outs["ozaki"], outs["simt"]) < tol
    assert abs(enls["ozaki"] - enls["simt"]) <= tol * abs(enls["simt"])


def test_hpsi_pieces_local_only_and_no_states(cuda):
    cell = synth.make_cell("t12b")
    b = Q.Basis(cell.L, cell.ecut)
    H = Q.Hamiltonian(b, *cell.grid)
    v = synth.vlocal(cell)
    H.set_vlocal(v)
    psi = synth.wavefunctions(cell, b)
    ob = O.Basis(b.a, cell.ecut)
    oft = O.FT(ob, *cell.grid)
    oh = O.Ham(oft, v, [])
    torch = _torch()
    out = torch.zeros_like(dev(psi))
    H.hpsi(dev(psi), out, synth.occupations(cell))
    ref, _ = oh.hpsi(psi.T, synth.occupations(cell))
    assert rel_err(out.cpu().numpy(), ref.T) < 1e-10
    # nst = 0 is a no-op
    H.hpsi(dev(psi), out, synth.occupations(cell), nst=0)


def test_density_and_current_vs_oracle(cuda):
    cell, b, H, oft, oh, psi = setup("c1")
    occ = synth.occupations(cell)
    torch = _torch()
    rho = torch.zeros(oft.n012, dtype=torch.float64, device=cuda)
    nel = H.update_density(dev(psi), occ, rho)
    rref, nref = O.update_density(oft, psi.T, occ)
    assert rel_err(rho.cpu().numpy(), rref) < 1e-12
    assert abs(nel - nref) < 1e-10 * nref
    assert abs(nel - occ.sum()) < 1e-8
    A = synth.kick()
    H.set_vector_potential(A)
    J = H.current(dev(psi), occ, nel)
    Jg = O.current_g(O.Basis(b.a, cell.ecut), psi.T, occ, A, nref)
    Jr = O.current_rs(oft, psi.T, occ, A, nref)
    assert np.abs(J - Jg).max() < 1e-10 * max(1.0, np.abs(Jg).max())
    assert np.abs(J - Jr).max() < 1e-9 * max(1.0, np.abs(Jr).max())


@pytest.mark.parametrize("nsteps", [1, 3])
def test_etrs_fp64_vs_oracle(cuda, nsteps):
    cell, b, H, oft, oh, psi = setup("t12")
    occ = synth.occupations(cell)
    A = synth.kick()
    dt = 0.05
    torch = _torch()
    p = dev(psi)
    rho = torch.zeros(oft.n012, dtype=torch.float64, device=cuda)
    ref = psi.T.copy()
    oh.set_A(A)
    for _ in range(nsteps):
        nel = H.etrs_step(p, occ, dt, A_t=A, A_tdt=A, rho=rho, want_nel=True)
        ref, rref, nref = oh.etrs_step(ref, occ, dt, A, A, want_rho=True, nthreads=NT)
    assert rel_err(p.cpu().numpy(), ref.T) < 1e-10
    assert rel_err(rho.cpu().numpy(), rref) < 1e-10
    assert abs(nel - nref) < 1e-10 * nref


def test_etrs_time_dependent_vector_potential(cuda):
    cell, b, H, oft, oh, psi = setup("t12b")
    occ = synth.occupations(cell)
    dt = 0.05
    torch = _torch()
    p = dev(psi)
    ref = psi.T.copy()
    for k in range(2):
        A0 = np.array([0.0, 0.02 * k, 0.01 + 0.005 * k])
        A1 = np.array([0.0, 0.02 * (k + 1), 0.01 + 0.005 * (k + 1)])
        H.etrs_step(p, occ, dt, A_t=A0, A_tdt=A1)
        ref, _, _ = oh.etrs_step(ref, occ, dt, A0, A1, nthreads=NT)
    assert rel_err(p.cpu().numpy(), ref.T) < 1e-10


@pytest.mark.parametrize("name,prec", [("t12", "mixed"), ("c1", "mixed"), ("c1", "mixed_fft64"),
                                       ("c1", "mixed_df32"), ("t12b", "mixed_nl64")])
def test_hpsi_mixed_vs_oracle(cuda, name, prec):
    """Reduced-precision forms (tensor-core projector GEMMs with a 2-piece FP16
    split and/or FP32 or double-float transforms; FP64 kinetic term and FP64
    in/out): <= 2e-6 relative to the FP64 oracle."""
    cell, b, H, oft, oh, psi = setup(name, prec=prec)
    occ = synth.occupations(cell)
    torch = _torch()
    out = torch.zeros_like(dev(psi))
    enl = H.hpsi(dev(psi), out, occ, want_enl=True)
    ref, enl_ref = oh.hpsi(psi.T, occ, nthreads=NT)
    err = rel_err(out.cpu().numpy(), ref.T)
    assert err < 2e-6, err
    assert abs(enl - enl_ref) <= 2e-6 * abs(enl_ref)
    # the nonlocal part alone through the tensor cores
    parts, _ = oh.parts(psi.T, occ, nthreads=NT)
    Hloc = Q.Hamiltonian(b, *cell.grid, precision=prec)
    Hloc.set_vlocal(np.zeros(oft.n012))
    Hloc.set_nonlocal(synth.species(cell))
    out2 = torch.zeros_like(out)
    Hloc.hpsi(dev(psi), out2, occ)
    nl_ref = parts[0].T + parts[1].T  # nonlocal + kinetic (v = 0)
    assert rel_err(out2.cpu().numpy(), nl_ref) < 2e-6


def test_etrs_mixed_error_vs_fp64_oracle(cuda):
    cell, b, H, oft, oh, psi = setup("t12", prec="mixed")
    occ = synth.occupations(cell)
    A = synth.kick()
    torch = _torch()
    p = dev(psi)
    ref = psi.T.copy()
    for _ in range(3):
        H.etrs_step(p, occ, 0.05, A_t=A, A_tdt=A)
        ref, _, _ = oh.etrs_step(ref, occ, 0.05, A, A, nthreads=NT)
    err = rel_err(p.cpu().numpy(), ref.T)
    assert err < 5e-5, err


def test_unsupported_and_too_small_grids(cuda):
    b = Q.Basis(12.0, 10.0)
    with pytest.raises(Q.QbgError, match="unsupported"):
        Q.FourierTransform(b, 34, 32, 32)   # 34 = 2*17
    with pytest.raises(Q.QbgError, match="invalid"):
        Q.FourierTransform(b, 16, 16, 16)   # sphere does not fit


def test_df32_transforms_match_fp64_closely(cuda):
    """The double-float transforms carry ~48 bits: the local part of H psi
    agrees with the FP64 form to ~1e-12."""
    cell = synth.make_cell("c1")
    b = Q.Basis(cell.L, cell.ecut)
    v = synth.vlocal(cell)
    psi = synth.wavefunctions(cell, b)
    outs = {}
    torch = _torch()
    for prec in ("fp64", "mixed_df32"):
        H = Q.Hamiltonian(b, *cell.grid, precision=prec)
        H.set_vlocal(v)
        o = torch.zeros_like(dev(psi))
        H.hpsi(dev(psi), o, synth.occupations(cell))
        outs[prec] = o.cpu().numpy()
    assert rel_err(outs["mixed_df32"], outs["fp64"]) < 1e-11


def species_fixture():
    """Projector tables of two pseudopotentials of the reference's own test
    suite (ONCV Xe from UPF, ONCV Ar from QSO XML; s, p, d, two channels),
    made by the reference's Species code (tests/golden/make_golden.py)."""
    from conftest import load_golden
    g = load_golden("species_xe_ar")
    sp = [dict(tau=g[f"tau{i}"], twnl=g[f"twnl{i}"], lproj=g[f"lproj{i}"], wt=g[f"wt{i}"])
          for i in range(len(g["names"]))]
    return g, sp


@pytest.mark.parametrize("prec,gemm,tol", [("fp64", "ozaki", 1e-10), ("fp64", "simt", 1e-10),
                                           ("mixed_df32", None, 2e-6)])
def test_hpsi_and_etrs_real_pseudopotential_tables(cuda, prec, gemm, tol):
    """H|psi> and one ETRS step with the projector tables of real
    pseudopotentials passed through qbg_set_nonlocal_tables, against the
    oracle fed the identical tables (26 projectors per Xe + Ar pair)."""
    g, sp = species_fixture()
    b = Q.Basis(g["a"], float(g["ecut"]))
    grid = tuple(int(x) for x in g["grid"])
    A = np.asarray(g["A"])
    H = Q.Hamiltonian(b, *grid, precision=prec)
    if gemm:
        H.set_fp64_gemm(gemm)
    cell = synth.make_cell("t12")
    v = synth.vlocal(cell)
    H.set_vlocal(v)
    H.set_vector_potential(A)
    H.set_nonlocal(sp)
    oft = O.FT(O.Basis(b.a, float(g["ecut"])), *grid)
    oh = O.Ham(oft, v, sp)
    oh.set_A(A)
    psi = synth.wavefunctions(cell, b, nst=6)
    occ = np.full(6, 2.0)
    torch = _torch()
    out = torch.zeros_like(dev(psi))
    enl = H.hpsi(dev(psi), out, occ, want_enl=True)
    ref, enl_ref = oh.hpsi(psi.T, occ, nthreads=NT)
    assert rel_err(out.cpu().numpy(), ref.T) < tol
    assert abs(enl - enl_ref) <= tol * abs(enl_ref)
    p = dev(psi)
    H.etrs_step(p, occ, 0.05)
    ref2, _, _ = oh.etrs_step(psi.T.copy(), occ, 0.05, A, A, nthreads=NT)
    assert rel_err(p.cpu().numpy(), ref2.T) < (tol if prec == "fp64" else 5e-5)


@pytest.mark.parametrize("name,kw", [("c1", {}), ("c2", dict(natoms=8, nst=40))])
def test_gram_vs_oracle(cuda, name, kw):
    """SlaterDet::gram on the device (FP64 overlap and product, host
    Cholesky) against the oracle's restatement on the same seeded
    non-orthogonal states, with a padded leading dimension."""
    cell = synth.make_cell(name, **kw)
    b = Q.Basis(cell.L, cell.ecut)
    H = Q.Hamiltonian(b, *cell.grid)
    rng = np.random.default_rng(3)
    n = cell.nst
    c = (rng.standard_normal((n, b.ngw)) + 1j * rng.standard_normal((n, b.ngw))) \
        * np.exp(-b.kpg2 / 8)[None, :]
    ld = b.ngw + 5
    cp = np.zeros((n, ld), complex)
    cp[:, :b.ngw] = c
    cp[:, b.ngw:] = 9.0
    torch = _torch()
    p = dev(cp)
    H.gram(p, ld=ld)
    out = p.cpu().numpy()
    ref = O.gram(c.T).T
    assert rel_err(out[:, :b.ngw], ref) < 1e-12
    ov = out[:, :b.ngw].conj() @ out[:, :b.ngw].T
    assert np.abs(ov - np.eye(n)).max() < 1e-12
    assert np.all(out[:, b.ngw:] == 9.0)
