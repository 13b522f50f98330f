"""Host arithmetic of the dipole-loss gradients (no GPU): the loss and its
derivative with respect to the step currents, the pulse integrals behind
A(t) and the chain to the pulse amplitudes, each against finite differences
or quadrature."""
import numpy as np
from scipy import integrate

from qball_gb300 import adjoint as ad


def test_loss_derivative_matches_finite_differences():
    rng = np.random.default_rng(3)
    N, dt = 7, 0.05
    J = rng.standard_normal((N + 1, 3))
    dstar = ad.target_dipole(N)
    L0, gJ = ad.loss_and_dJ(J, dt, dstar)
    h = 1e-6
    for n in range(N + 1):
        for d in range(3):
            Jp, Jm = J.copy(), J.copy()
            Jp[n, d] += h
            Jm[n, d] -= h
            fd = (ad.loss_and_dJ(Jp, dt, dstar)[0] - ad.loss_and_dJ(Jm, dt, dstar)[0]) / (2 * h)
            assert abs(fd - gJ[n, d]) < 1e-7 * max(1.0, abs(fd)), (n, d, fd, gJ[n, d])


def test_pulse_integrals_match_quadrature():
    times = 0.05 * np.arange(41)
    tk, ak, sigma = ad.pulse_train(5, times[-1], seed=2)
    G = ad.pulse_integrals(times, tk, sigma)
    for n in (0, 7, 40):
        for k in range(5):
            q, _ = integrate.quad(lambda s: np.exp(-(s - tk[k]) ** 2 / (2 * sigma ** 2)), 0.0,
                                  times[n], epsabs=1e-14, epsrel=1e-13)
            assert abs(G[n, k] - q) < 1e-12


def test_amplitude_chain_matches_finite_differences():
    """A linear-quadratic stand-in for the device map a_n -> L checks
    grad_amplitudes and vector_potential together."""
    rng = np.random.default_rng(4)
    N, nk = 12, 6
    times = 0.1 * np.arange(N + 1)
    tk, ak, sigma = ad.pulse_train(nk, times[-1], seed=8)
    G = ad.pulse_integrals(times, tk, sigma)
    e = np.array([0.0, 0.6, 0.8])
    W = rng.standard_normal((N + 1, 3))

    def loss(a):
        A = ad.vector_potential(a, G, e, A0=(0.0, 0.0, 0.01))
        return float(np.sum(W * A) + np.sum(A ** 2))

    A = ad.vector_potential(ak, G, e, A0=(0.0, 0.0, 0.01))
    grad_a = (W + 2 * A) @ e  # dL/da_n along e
    g = ad.grad_amplitudes(grad_a, G)
    h = 1e-6
    for k in range(nk):
        ap, am = ak.copy(), ak.copy()
        ap[k] += h
        am[k] -= h
        fd = (loss(ap) - loss(am)) / (2 * h)
        assert abs(fd - g[k]) < 1e-7 * max(1.0, abs(fd))
