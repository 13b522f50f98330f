"""CPU restatement of the adjoint of the fixed-potential ETRS step.

Test infrastructure only: tests import it as the checker of the product's
adjoint (qbg_td_*, qbg_etrs_adjoint_step); the product library never calls
it.  It runs on the oracle's own operators (oracle.Ham, oracle.FT, the
G-space current), all FP64, with every state of a run kept in memory (no
checkpoints: the runs it checks are a few steps of a small cell).

The step is psi_{n+1} = P_b P_a psi_n, P = sum_{k<=4} c_k H^k,
c_k = (-i tau)^k / k!, tau = dt/2 (ExponentialWavefunctionStepper.cc:98-126);
with dL = 2 Re sum <lambda|d psi>:
  lambda_n = P_a^+ P_b^+ lambda_{n+1} + dL/dpsi_n*,
  dL/dtheta += 2 Re sum_m <M_m|dH/dtheta|H^m x0>,  M_m = sum_j conj(c_{j+m+1}) H^j y0,
  dL/dv(r)  = (2/N) Re sum_m conj(M_m(r)) (H^m x0)(r),
  dH/da     = -(k+G-A).e  +  sum_p (D_p/Omega) (|b'_p><b_p| + |b_p><b'_p|).
The projector derivative b' along e is taken from the oracle's own projector
table (NonLocalPotential.cc:1962-2037 restated in qbo.c) by fourth-order
central differences in A (h = 2e-4, error ~1e-11), independently of the
product's analytic derivative.
"""
import numpy as np

from oracle import oracle as O


def taylor_coefs(tau):
    c = [1.0 + 0.0j]
    for k in range(1, 5):
        c.append(c[-1] * (-1j * tau / k))
    return c


class TDAdjoint:
    """Forward and adjoint of nsteps fixed-potential ETRS steps on the oracle.

    basis: oracle.Basis; ft: oracle.FT; v_r: local potential; species: the
    oracle.Ham species list; occ: occupations; psi: [ngw, nst]."""

    def __init__(self, basis, ft, v_r, species, occ, dt):
        self.basis, self.ft = basis, ft
        self.ham = O.Ham(ft, v_r, species)
        self.occ = np.asarray(occ, float)
        self.nel = float(self.occ.sum())
        self.dt = dt
        self.P = self.ham.nproj()
        self.wt = np.array([self.ham.projector(p)[2] for p in range(self.P)]) / basis.omega

    def H(self, x):
        return self.ham.hpsi(x, self.occ)[0]

    def forward(self, psi0, A):
        """States psi_0..psi_N and currents J_0..J_N (A: [(N+1), 3])."""
        N = len(A) - 1
        states = [np.asfortranarray(psi0)]
        J = [O.current_g(self.basis, psi0, self.occ, A[0], self.nel)]
        for n in range(N):
            psi, _, _ = self.ham.etrs_step(states[-1], self.occ, self.dt, A[n], A[n + 1])
            states.append(psi)
            J.append(O.current_g(self.basis, psi, self.occ, A[n + 1], self.nel))
        return states, np.array(J)

    def table(self, A):
        """anl[p][g] = twnl (-i)^l exp(-i (k+G-A).tau) at A (qbo.c anl column)."""
        self.ham.set_A(A)
        q = self.basis.kpgx.reshape(3, -1) - np.asarray(A, float)[:, None]
        out = np.empty((self.P, q.shape[1]), complex)
        for p in range(self.P):
            t, l, _, tau = self.ham.projector(p)
            out[p] = t * (-1j) ** l * np.exp(-1j * (tau @ q))
        return out

    def dtable(self, A, e, h=2e-4):
        A, e = np.asarray(A, float), np.asarray(e, float)
        f = {s: self.table(A + s * h * e) for s in (-2, -1, 1, 2)}
        self.ham.set_A(A)
        return (8.0 * (f[1] - f[-1]) - (f[2] - f[-2])) / (12.0 * h)

    def factor(self, x0, y0, tau, A, e):
        """(P^+ y0, dL/dv contribution, dL/da contribution) of one factor at A."""
        self.ham.set_A(A)
        c = taylor_coefs(tau)
        cc = [np.conj(v) for v in c]
        X = [x0]
        for _ in range(3):
            X.append(self.H(X[-1]))
        Y = [y0]
        for _ in range(4):
            Y.append(self.H(Y[-1]))
        y_next = sum(cc[k] * Y[k] for k in range(5))
        M = [sum(cc[j + m + 1] * Y[j] for j in range(4 - m)) for m in range(4)]
        N = self.ft.n012
        gv = np.zeros(N)
        for m in range(4):
            for s in range(x0.shape[1]):
                gv += (2.0 / N) * np.real(np.conj(self.ft.backward(M[m][:, s])) *
                                          self.ft.backward(X[m][:, s]))
        q = self.basis.kpgx.reshape(3, -1) - np.asarray(A, float)[:, None]
        d = -(np.asarray(e, float) @ q)
        ga = 0.0
        for m in range(4):
            ga += 2.0 * np.real(np.sum(np.conj(M[m]) * d[:, None] * X[m]))
        if self.P:
            b = self.table(A)
            db = self.dtable(A, e)
            for m in range(4):
                bM, bX = b.conj() @ M[m], b.conj() @ X[m]
                dM, dX = db.conj() @ M[m], db.conj() @ X[m]
                ga += 2.0 * np.real(np.sum(self.wt[:, None] * (np.conj(dM) * bX + np.conj(bM) * dX)))
        return y_next, gv, ga

    def step_adjoint(self, psi_n, lam, A_n, A_np1, e):
        """lambda_n (before the direct term), dL/dv and [dL/da_n, dL/da_{n+1}]."""
        tau = 0.5 * self.dt
        self.ham.set_A(A_n)
        c = taylor_coefs(tau)
        phi = psi_n.copy()
        x = psi_n
        for k in range(1, 5):
            x = self.H(x)
            phi = phi + c[k] * x
        chi, gv_b, ga_b = self.factor(phi, lam, tau, A_np1, e)
        lam_n, gv_a, ga_a = self.factor(psi_n, chi, tau, A_n, e)
        return lam_n, gv_a + gv_b, np.array([ga_a, ga_b])

    def backward(self, states, A, dLdJ, e):
        """dL/dv(r), dL/da_n (along e) and lambda_0 for a loss of the currents."""
        N = len(states) - 1
        kp = self.basis.kpgx.reshape(3, -1)
        e = np.asarray(e, float)

        def direct(n):
            g = dLdJ[n]
            return -(g @ kp)[:, None] * self.occ[None, :] * states[n]

        gv = np.zeros(self.ft.n012)
        ga = np.array([self.nel * float(dLdJ[n] @ e) for n in range(N + 1)])
        lam = direct(N)
        for n in range(N - 1, -1, -1):
            lam, dv, da = self.step_adjoint(states[n], lam, A[n], A[n + 1], e)
            gv += dv
            ga[n] += da[0]
            ga[n + 1] += da[1]
            lam = lam + direct(n)
        return gv, ga, lam
