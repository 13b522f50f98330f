"""The oracle's Hartree + LDA update (CPU).

Pins: the LDA restatement equals the reference's own LDAFunctional::setxc
bit for bit (golden vectors from oracle/_ref, tests/golden/ref_lda.npz).
Identities: v_xc = d(rho e_xc)/d rho; the Hartree and ionic energies
summed in G space equal their real-space integrals (Parseval, exact for a
density band-limited to the density sphere); the self-consistent ETRS step
conserves the electron count and really feeds the density back into v_r.
"""
import numpy as np
import pytest

from oracle import oracle as O
from qball_gb300 import synth

from conftest import load_golden


def test_lda_matches_reference_bitwise():
    g = load_golden("lda")
    e, v = O.lda(g["rho"])
    assert np.array_equal(e, g["exc"])
    assert np.array_equal(v, g["vxc"])


def test_lda_reference_pin_live():
    if O.ref() is None:
        pytest.skip("oracle/_ref not built")
    rho = np.random.default_rng(3).uniform(0.0, 2.0, 300)
    e, v = O.lda(rho)
    er, vr = O.ref_lda(rho)
    assert np.array_equal(e, er) and np.array_equal(v, vr)


@pytest.mark.parametrize("rho", [1e-4, 1e-2, 0.05, 0.2, 3.0 / (4.0 * np.pi), 0.5, 5.0])
def test_lda_potential_is_energy_derivative(rho):
    h = 1e-5 * rho
    ep, _ = O.lda([rho + h])
    em, _ = O.lda([rho - h])
    _, v = O.lda([rho])
    dfdr = ((rho + h) * ep[0] - (rho - h) * em[0]) / (2 * h)
    assert abs(dfdr - v[0]) < 1e-7 * abs(v[0])


@pytest.fixture(scope="module")
def cell12():
    """t12 cell on the reference's grid for the 4 ecut density basis (40^3)."""
    cell = synth.make_cell("t12", grid=(40, 40, 40))
    a = np.diag([cell.L] * 3).reshape(9)
    assert synth.rule_grid(cell.L, 4 * cell.ecut) == 40
    b = O.Basis(a, cell.ecut)
    vb = O.Basis(a, 4 * cell.ecut)
    ft = O.FT(b, *cell.grid)
    vion, rhopst = synth.ionic_terms(cell, vb)
    hxc = O.Hxc(vb, *cell.grid, vion, rhopst)
    psi = synth.wavefunctions(cell, b)
    occ = synth.occupations(cell)
    rho, nel = O.update_density(ft, psi.T, occ)
    return cell, b, vb, ft, hxc, psi, occ, rho, nel


def test_density_g_is_charge(cell12):
    cell, b, vb, ft, hxc, psi, occ, rho, nel = cell12
    rg = hxc.density_g(rho)
    # rho_G(0) = Omega * mean(rho) = electron count (rod (0,0) first, l ascending)
    i0 = int(np.flatnonzero(vb.kpg2 == 0.0)[0])
    assert abs(rg[i0].real - nel) < 1e-10 * nel
    assert abs(nel - 2.0 * cell.nst) < 1e-9 * nel
    # band-limited: the density basis round trip reproduces rho
    back = hxc.vft.backward(rg / vb.omega).real
    assert np.abs(back - rho).max() < 1e-12 * np.abs(rho).max()


def test_hartree_and_ionic_energies_parseval(cell12):
    cell, b, vb, ft, hxc, psi, occ, rho, nel = cell12
    v, en = hxc.update_vhxc(rho)
    N = ft.n012
    w = vb.omega / N
    _, vxc = O.lda(rho)
    v_ion = hxc.vft.backward(hxc.vion).real
    rho_ps = hxc.vft.backward(hxc.rhopst).real
    v_h = v - vxc - v_ion
    eh_r = 0.5 * w * np.dot(rho + rho_ps, v_h)
    assert abs(eh_r - en["ehart"]) < 1e-10 * abs(en["ehart"])
    assert abs(w * np.dot(rho, v_ion) - en["eps"]) < 1e-10 * abs(en["eps"])
    exc, _ = O.lda(rho)
    assert abs(w * np.dot(rho, exc) - en["exc"]) < 1e-12 * abs(en["exc"])
    # v_H has no G = 0 component and the cell is neutral
    assert abs(v_h.mean()) < 1e-10 * np.abs(v_h).max()
    i0 = int(np.flatnonzero(vb.kpg2 == 0.0)[0])
    assert abs(hxc.density_g(rho_ps)[i0].real + nel) < 1e-9 * nel


def test_etrs_selfconsistent_conserves_charge_and_couples(cell12):
    cell, b, vb, ft, hxc, psi, occ, rho, nel = cell12
    v0, _ = hxc.update_vhxc(rho)
    ham = O.Ham(ft, v0, synth.species(cell))
    A = synth.kick()
    p1, rho1, nel1 = ham.etrs_step_hxc(psi.T, occ, 0.05, A, A, hxc, want_rho=True, nthreads=4)
    assert abs(nel1 - nel) < 1e-5 * nel
    # norm of every state kept to O(dt^5)
    nrm = np.einsum("gi,gi->i", p1.conj(), p1).real
    assert np.abs(nrm - 1.0).max() < 1e-6
    # the potential in use after the step is the one of the predicted density
    v1, _ = hxc.update_vhxc(rho1)
    assert np.array_equal(ham.v_r_now(), v1)
    # and the fixed-potential step differs from the self-consistent one
    ham2 = O.Ham(ft, v0, synth.species(cell))
    p2, _, _ = ham2.etrs_step(psi.T, occ, 0.05, A, A, nthreads=4)
    assert np.abs(p2 - p1).max() > 1e-8


def test_oracle_aetrs_fixed_potential_equals_etrs():
    """With a fixed potential and a constant A, the extrapolated potential is
    the potential itself and the predictor changes nothing: the oracle's AETRS
    steps equal its ETRS steps bit for bit."""
    import qball_gb300 as Q
    from qball_gb300 import synth
    from oracle import oracle as O
    cell = synth.make_cell("t12b")
    b = O.Basis(Q.cubic_cell(cell.L), cell.ecut)
    ft = O.FT(b, *cell.grid)
    v = synth.vlocal(cell)
    rng = np.random.default_rng(2)
    c = (rng.standard_normal((b.ngw, 3)) + 1j * rng.standard_normal((b.ngw, 3))) \
        * np.exp(-b.kpg2 / 8)[:, None]
    c = O.gram(c)
    occ = np.full(3, 2.0)
    A = synth.kick()
    h1 = O.Ham(ft, v, synth.species(cell))
    h2 = O.Ham(ft, v, synth.species(cell))
    h1.set_A(A)
    h2.set_A(A)
    x1, x2 = c.copy(), c.copy()
    for _ in range(4):
        x1, _, _ = h1.etrs_step(x1, occ, 0.05, A, A)
        x2 = h2.aetrs_step(x2, occ, 0.05, A, A)
    assert np.array_equal(x1, x2)
