"""The oracle's adjoint of the fixed-potential ETRS step (CPU): its gradients
against central finite differences of the oracle's own forward (the restated
ExponentialWavefunctionStepper and G-space current), for a dipole loss over
a short laser-driven run of the 12-bohr cell; its one-step adjoint identity;
its projector derivative against the analytic form the product uses."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle.adjoint import TDAdjoint
from qball_gb300 import adjoint as ad
from qball_gb300 import synth

DT = 0.05
E = np.array([0.0, 0.0, 1.0])
NST = 3


@pytest.fixture(scope="module")
def run():
    cell = synth.make_cell("t12")
    a = np.diag([cell.L] * 3).reshape(9)
    b = O.Basis(a, cell.ecut)
    ft = O.FT(b, *cell.grid)
    v = synth.vlocal(cell)
    psi = np.asfortranarray(synth.wavefunctions(cell, b, nst=NST).T)
    occ = synth.occupations(cell, nst=NST)
    N = 3
    times = DT * np.arange(N + 1)
    tk, ak, sigma = ad.pulse_train(3, times[-1], seed=21, amp=0.05)
    G = ad.pulse_integrals(times, tk, sigma)
    return cell, b, ft, v, psi, occ, ak, G, N


def _loss(cell, b, ft, v, psi, occ, ak, G, dstar):
    td = TDAdjoint(b, ft, v, synth.species(cell), occ, DT)
    A = ad.vector_potential(ak, G, E, A0=synth.kick())
    _, J = td.forward(psi, A)
    return ad.loss_and_dJ(J, DT, dstar)[0]


def test_oracle_adjoint_matches_finite_differences(run):
    cell, b, ft, v, psi, occ, ak, G, N = run
    dstar = ad.target_dipole(N, scale=2e-3)
    td = TDAdjoint(b, ft, v, synth.species(cell), occ, DT)
    A = ad.vector_potential(ak, G, E, A0=synth.kick())
    states, J = td.forward(psi, A)
    L, gJ = ad.loss_and_dJ(J, DT, dstar)
    gv, ga, _ = td.backward(states, A, gJ, E)
    gk = ad.grad_amplitudes(ga, G)
    dv = 0.1 * np.random.default_rng(17).standard_normal(v.shape)
    h = 1e-4
    fd = (_loss(cell, b, ft, v + h * dv, psi, occ, ak, G, dstar) -
          _loss(cell, b, ft, v - h * dv, psi, occ, ak, G, dstar)) / (2 * h)
    assert abs(fd - gv @ dv) < 1e-6 * abs(fd), (fd, gv @ dv)
    h = 1e-5
    for k in range(len(ak)):
        ap, am = ak.copy(), ak.copy()
        ap[k] += h
        am[k] -= h
        fd = (_loss(cell, b, ft, v, psi, occ, ap, G, dstar) -
              _loss(cell, b, ft, v, psi, occ, am, G, dstar)) / (2 * h)
        assert abs(fd - gk[k]) < 1e-6 * max(abs(fd), 1e-3 * np.abs(gk).max()), (k, fd, gk[k])


def test_oracle_step_adjoint_identity(run):
    cell, b, ft, v, psi, occ, ak, G, N = run
    td = TDAdjoint(b, ft, v, synth.species(cell), occ, DT)
    rng = np.random.default_rng(9)
    x = rng.standard_normal(psi.shape) + 1j * rng.standard_normal(psi.shape)
    lam = rng.standard_normal(psi.shape) + 1j * rng.standard_normal(psi.shape)
    A0, A1 = np.array([0.0, 0.0, 0.01]), np.array([0.003, -0.002, 0.02])
    y, _, _ = td.ham.etrs_step(x, occ, DT, A0, A1)
    l2, _, _ = td.step_adjoint(np.asfortranarray(x), lam, A0, A1, E)
    lhs, rhs = np.vdot(lam, y), np.vdot(l2, x)
    assert abs(lhs - rhs) < 1e-12 * abs(lhs)


def _solid(l, q):
    """(s_l, [(P_lm(q), grad P_lm(q))] for m = 0..2l) of the synthetic form."""
    qx, qy, qz = q
    z, o = np.zeros_like(qx), np.ones_like(qx)
    fpi = 4.0 * np.pi
    if l == 0:
        return np.sqrt(1 / fpi), [(o, (z, z, z))]
    if l == 1:
        return np.sqrt(3 / fpi), [(qx, (o, z, z)), (qy, (z, o, z)), (qz, (z, z, o))]
    s3 = np.sqrt(3.0)
    return np.sqrt(5 / fpi), [
        (0.5 * (2 * qz * qz - qx * qx - qy * qy), (-qx, -qy, 2 * qz)),
        (0.5 * s3 * (qx * qx - qy * qy), (s3 * qx, -s3 * qy, z)),
        (s3 * qx * qy, (s3 * qy, s3 * qx, z)),
        (s3 * qy * qz, (z, s3 * qz, s3 * qy)),
        (s3 * qx * qz, (s3 * qz, z, s3 * qx))]


def test_oracle_projector_derivative_matches_analytic_form(run):
    """The oracle's table differenced in A against the closed-form derivative
    that k_anl_da evaluates: d/da [kappa_l s_l P_lm(q) exp(-|q|^2 rc^2/2)
    exp(-i q.tau)] = -kappa_l exp(-i q.tau) (e.grad t - i (e.tau) t)."""
    cell, b, ft, v, psi, occ, ak, G, N = run
    td = TDAdjoint(b, ft, v, synth.species(cell), occ, DT)
    A = np.array([0.01, -0.02, 0.03])
    e = np.array([0.6, 0.0, 0.8])
    db = td.dtable(A, e)
    td.ham.set_A(A)
    q = b.kpgx.reshape(3, -1) - A[:, None]
    rc = synth.species(cell)[0]["rc"]
    E_ = np.exp(-0.5 * np.sum(q * q, axis=0) * rc * rc)
    eq = e @ q
    for p in range(td.P):
        t_or, l, _, tau = td.ham.projector(p)
        s_l, cands = _solid(l, q)
        # the m of this projector: the candidate the oracle's table equals
        errs = [np.abs(s_l * P * E_ - t_or).max() for P, _ in cands]
        m = int(np.argmin(errs))
        assert errs[m] < 1e-12 * max(1.0, np.abs(t_or).max())
        P, gP = cands[m]
        t = s_l * P * E_
        et = s_l * E_ * (e[0] * gP[0] + e[1] * gP[1] + e[2] * gP[2] - rc * rc * P * eq)
        kappa = (-1j) ** l
        d_an = -kappa * np.exp(-1j * (tau @ q)) * (et - 1j * (e @ tau) * t)
        assert np.abs(d_an - db[p]).max() < 1e-9 * max(np.abs(db[p]).max(), 1e-30), p
