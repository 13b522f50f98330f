"""Identities the oracle restatement must satisfy (CPU, small cells).

These complement the bit-exact pins of the transforms: H is Hermitian, the
current computed in real space (the reference's CurrentDensity route) equals
its G-space Parseval form, the density integrates to the electron count, and
the 4th-order Taylor ETRS step conserves the norm to O(dt^5).
"""
import numpy as np
import pytest

from oracle import oracle as O
from qball_gb300 import synth


@pytest.fixture(scope="module")
def small():
    cell = synth.make_cell("t12")
    b = O.Basis(np.diag([cell.L] * 3).reshape(9), cell.ecut)
    ft = O.FT(b, *cell.grid)
    v = synth.vlocal(cell)
    ham = O.Ham(ft, v, synth.species(cell))
    psi = synth.wavefunctions(cell, b)
    return cell, b, ft, ham, psi


def test_hamiltonian_is_hermitian(small):
    cell, b, ft, ham, psi = small
    ham.set_A(synth.kick())
    hp, enl = ham.hpsi(psi.T, synth.occupations(cell))
    m = psi.conj() @ hp
    assert np.abs(m - m.conj().T).max() < 1e-12 * np.abs(m).max()
    assert enl > 0


def test_hpsi_is_sum_of_parts(small):
    cell, b, ft, ham, psi = small
    occ = synth.occupations(cell)
    hp, _ = ham.hpsi(psi.T, occ)
    (nl, kin, loc), _ = ham.parts(psi.T, occ)
    assert np.abs(hp - (nl + kin + loc)).max() < 1e-13 * np.abs(hp).max()


def test_density_integrates_to_electron_count(small):
    cell, b, ft, ham, psi = small
    occ = synth.occupations(cell)
    rho, nel = O.update_density(ft, psi.T, occ)
    assert abs(nel - occ.sum()) < 1e-10
    assert rho.min() >= 0.0


def test_current_real_space_equals_parseval(small):
    cell, b, ft, ham, psi = small
    occ = synth.occupations(cell)
    A = np.array([0.003, -0.002, 0.01])
    Jr = O.current_rs(ft, psi.T, occ, A, occ.sum())
    Jg = O.current_g(b, psi.T, occ, A, occ.sum())
    assert np.abs(Jr - Jg).max() < 1e-11 * max(1.0, np.abs(Jg).max())


def test_etrs_conserves_norm_and_charge(small):
    cell, b, ft, ham, psi = small
    occ = synth.occupations(cell)
    A = synth.kick()
    ham.set_A(A)
    out, rho, nel = ham.etrs_step(psi.T.copy(), occ, 0.05, A, A, want_rho=True, nthreads=4)
    ov = out.conj().T @ out
    # the truncated Taylor series is unitary to O(dt^5); nel is the charge of
    # the predicted psi(t+dt), built with two exponentials
    assert np.abs(ov - np.eye(cell.nst)).max() < 1e-6
    assert abs(nel - occ.sum()) < 1e-5 * occ.sum()


def test_etrs_small_dt_matches_exact_propagator(small):
    """With v = 0 and no projectors H is diagonal in G (0.5|k+G-A|^2), so
    exp(-i H dt) is exact and the ETRS step must reproduce it to the Taylor
    truncation error."""
    cell, b, ft, _, psi = small
    ham0 = O.Ham(ft, np.zeros(ft.n012), [])
    A = np.array([0.0, 0.0, 0.02])
    ham0.set_A(A)
    dt = 0.01
    out, _, _ = ham0.etrs_step(psi.T.copy(), synth.occupations(cell), dt, A, A)
    kx = b.kpgx.reshape(3, -1)
    e = 0.5 * ((kx[0] - A[0]) ** 2 + (kx[1] - A[1]) ** 2 + (kx[2] - A[2]) ** 2)
    exact = np.exp(-1j * e * dt)[:, None] * psi.T
    assert np.abs(out - exact).max() < 1e-9


def test_oracle_gram_orthonormalises_like_the_reference():
    """The oracle's SlaterDet::gram (C L^{-H}, C^H C = L L^H): orthonormal
    columns spanning the same space, L^H upper triangular (the first column
    only rescaled), and equal to the Cholesky row form of the seeded-state
    generator."""
    from oracle import oracle as O
    from qball_gb300 import synth
    rng = np.random.default_rng(4)
    c = rng.standard_normal((300, 12)) + 1j * rng.standard_normal((300, 12))
    x = O.gram(c)
    assert np.abs(x.conj().T @ x - np.eye(12)).max() < 1e-13
    t = np.linalg.lstsq(c, x, rcond=None)[0]  # x = c t, t upper triangular
    assert np.abs(np.tril(t, -1)).max() < 1e-12
    assert np.allclose(x[:, 0], c[:, 0] / np.linalg.norm(c[:, 0]), atol=1e-14)
    assert np.abs(x.T - synth.gram(c.T)).max() < 1e-13
