"""Adjoint of the fixed-potential ETRS step and the checkpointed operator pair.

- the operator pair's forward pass is the ETRS step (bitwise, currents too);
- the adjoint step is the adjoint of the step: <lam, S x> = <S^+ lam, x>
  (FP64, 1e-12);
- FP64 gradients equal the CPU oracle adjoint (oracle/adjoint.py, 1e-8);
- dL/dv(r) and dL/d(pulse amplitudes) of a dipole loss over a laser-driven
  run agree with central finite differences of the FP64 forward (1e-6);
- the gradients do not depend on the checkpoint interval (1e-13);
- on 120 x 120 planes the gradient paired inside the H applications equals
  the eight-field path (FP64 1e-12, mixed_df32 1e-10);
- the reduced-precision forms' gradients against the FP64 adjoint
  (mixed_df32 1e-8, mixed 1e-5; observed 1.2e-10 and 1.3e-7).
"""
import numpy as np
import pytest

from conftest import rel_err
import qball_gb300 as Q
from qball_gb300 import adjoint as ad
from qball_gb300 import synth

pytestmark = pytest.mark.gpu

DT = 0.05
E = np.array([0.0, 0.0, 1.0])


def _torch():
    import torch
    return torch


def dev(x):
    return _torch().from_numpy(np.ascontiguousarray(x)).to("cuda:0")


def setup(name, prec, **kw):
    cell = synth.make_cell(name, **kw)
    b = Q.Basis(cell.L, cell.ecut)
    H = Q.Hamiltonian(b, *cell.grid, precision=prec)
    v = synth.vlocal(cell)
    H.set_vlocal(v)
    H.set_nonlocal(synth.species(cell))
    psi = dev(synth.wavefunctions(cell, b))
    occ = synth.occupations(cell)
    return cell, H, v, psi, occ


def laser(nsteps, nk=4, amp=0.05):
    times = DT * np.arange(nsteps + 1)
    tk, ak, sigma = ad.pulse_train(nk, times[-1], seed=21, amp=amp)
    G = ad.pulse_integrals(times, tk, sigma)
    return ak, G


def potential(ak, G):
    return ad.vector_potential(ak, G, E, A0=synth.kick())


@pytest.mark.parametrize("prec", ["fp64", "mixed_df32"])
def test_forward_pass_is_the_etrs_step(cuda, prec):
    torch = _torch()
    N = 5
    cell, H, v, psi, occ = setup("t12", prec)
    ak, G = laser(N)
    A = potential(ak, G)
    td = Q.TDPropagation(H, psi, occ, DT, N, K=2)
    p = psi.clone()
    J = td.forward(p, A)
    _, H2, _, _, _ = setup("t12", prec)
    q = psi.clone()
    nel = float(np.sum(occ))
    H2.set_vector_potential(A[0])
    J2 = [H2.current(q, occ, nel)]
    for n in range(N):
        H2.etrs_step(q, occ, DT, A_t=A[n], A_tdt=A[n + 1])
        J2.append(H2.current(q, occ, nel))
    torch.cuda.synchronize()
    assert torch.equal(p, q)
    assert np.array_equal(J, np.array(J2))
    td.close()


def test_adjoint_step_is_the_adjoint(cuda):
    torch = _torch()
    cell, H, v, psi, occ = setup("t12", "fp64")
    rng = np.random.default_rng(9)
    shape = tuple(psi.shape)
    x = dev(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    lam = dev(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    A0, A1 = np.array([0.0, 0.0, 0.01]), np.array([0.003, -0.002, 0.02])
    y = x.clone()
    H.etrs_step(y, occ, DT, A_t=A0, A_tdt=A1)
    l2 = lam.clone()
    H.etrs_adjoint_step(x, l2, DT, A_n=A0, A_np1=A1)
    lhs = complex(torch.vdot(lam.flatten(), y.flatten()))
    rhs = complex(torch.vdot(l2.flatten(), x.flatten()))
    assert abs(lhs - rhs) < 1e-12 * abs(lhs), (lhs, rhs)


def _grads(H, psi, occ, ak, G, N, K, dstar):
    torch = _torch()
    td = Q.TDPropagation(H, psi, occ, DT, N, K=K)
    J = td.forward(psi.clone(), potential(ak, G))
    L, gJ = ad.loss_and_dJ(J, DT, dstar)
    gv = torch.zeros(H.n012, dtype=torch.float64, device="cuda:0")
    ga = td.backward(gJ, e=E, grad_v=gv)
    td.close()
    return L, gv.cpu().numpy(), ad.grad_amplitudes(ga, G)


def _loss(H, psi, occ, ak, G, N, dstar):
    td = Q.TDPropagation(H, psi, occ, DT, N, K=N)
    J = td.forward(psi.clone(), potential(ak, G))
    td.close()
    return ad.loss_and_dJ(J, DT, dstar)[0]


def test_gradients_match_finite_differences(cuda):
    N = 4
    cell, H, v, psi, occ = setup("t12", "fp64")
    ak, G = laser(N)
    dstar = ad.target_dipole(N, scale=2e-3)
    L, gv, gk = _grads(H, psi, occ, ak, G, N, 2, dstar)
    assert np.all(np.isfinite(gv)) and np.all(np.isfinite(gk))
    # local potential, along a random direction
    rng = np.random.default_rng(17)
    dv = 0.1 * rng.standard_normal(v.shape)
    h = 1e-4
    H.set_vlocal(v + h * dv)
    Lp = _loss(H, psi, occ, ak, G, N, dstar)
    H.set_vlocal(v - h * dv)
    Lm = _loss(H, psi, occ, ak, G, N, dstar)
    H.set_vlocal(v)
    fd = (Lp - Lm) / (2 * h)
    an = float(np.dot(gv, dv))
    assert abs(fd - an) < 1e-6 * abs(fd), (fd, an)
    # pulse amplitudes
    h = 1e-5
    for k in range(len(ak)):
        ap, am = ak.copy(), ak.copy()
        ap[k] += h
        am[k] -= h
        fd = (_loss(H, psi, occ, ap, G, N, dstar) - _loss(H, psi, occ, am, G, N, dstar)) / (2 * h)
        assert abs(fd - gk[k]) < 1e-6 * max(abs(fd), 1e-3 * np.abs(gk).max()), (k, fd, gk[k])


def test_gradients_do_not_depend_on_checkpoint_interval(cuda):
    N = 4
    cell, H, v, psi, occ = setup("t12", "fp64")
    ak, G = laser(N)
    dstar = ad.target_dipole(N, scale=2e-3)
    ref = _grads(H, psi, occ, ak, G, N, 1, dstar)
    for K in (3, 4):
        L, gv, gk = _grads(H, psi, occ, ak, G, N, K, dstar)
        assert L == ref[0]
        assert rel_err(gv, ref[1]) < 1e-13
        assert rel_err(gk, ref[2]) < 1e-13


@pytest.mark.parametrize("prec,tol", [("mixed_df32", 1e-8), ("mixed", 1e-5)])
def test_reduced_precision_gradients_vs_fp64_adjoint(cuda, prec, tol):
    N = 4
    ak, G = laser(N)
    dstar = ad.target_dipole(N, scale=2e-3)
    _, H64, _, psi, occ = setup("t12", "fp64")
    ref = _grads(H64, psi, occ, ak, G, N, 2, dstar)
    _, H, _, _, _ = setup("t12", prec)
    L, gv, gk = _grads(H, psi, occ, ak, G, N, 2, dstar)
    ev, ek = rel_err(gv, ref[1]), rel_err(gk, ref[2])
    print(f"{prec}: dL/dv rel err {ev:.2e}, dL/da_k rel err {ek:.2e}")
    assert ev < tol and ek < tol


def test_operator_pair_state_errors(cuda):
    cell, H, v, psi, occ = setup("t12", "fp64")
    with pytest.raises(Q.QbgError):
        Q.TDPropagation(H, psi, occ, DT, 0)
    td = Q.TDPropagation(H, psi, occ, DT, 2, K=1)
    with pytest.raises(Q.QbgError, match="no forward"):
        td.backward(np.zeros((3, 3)))
    td.close()


def test_gradients_match_oracle_adjoint(cuda):
    """FP64 operator pair against the CPU oracle's adjoint (oracle/adjoint.py)
    on the same seeded 3-state run of the 12-bohr cell."""
    from oracle import oracle as O
    from oracle.adjoint import TDAdjoint
    N, nst = 3, 3
    cell, H, v, _, _ = setup("t12", "fp64")
    b = Q.Basis(cell.L, cell.ecut)
    psi_h = synth.wavefunctions(cell, b, nst=nst)
    occ = synth.occupations(cell, nst=nst)
    ak, G = laser(N, nk=3)
    dstar = ad.target_dipole(N, scale=2e-3)
    L, gv, gk = _grads(H, dev(psi_h), occ, ak, G, N, 2, dstar)
    ob = O.Basis(b.a, cell.ecut)
    oft = O.FT(ob, *cell.grid)
    td = TDAdjoint(ob, oft, v, synth.species(cell), occ, DT)
    A = potential(ak, G)
    states, J = td.forward(np.asfortranarray(psi_h.T), A)
    Lo, gJ = ad.loss_and_dJ(J, DT, dstar)
    gvo, gao, _ = td.backward(states, A, gJ, E)
    gko = ad.grad_amplitudes(gao, G)
    assert abs(L - Lo) < 1e-10 * abs(Lo)
    assert rel_err(gv, gvo) < 1e-8, rel_err(gv, gvo)
    assert rel_err(gk, gko) < 1e-8, rel_err(gk, gko)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("mixed_df32", 1e-10)])
def test_whole_plane_gradient_matches_field_path(cuda, prec, tol):
    """dL/dv(r) on the 216-atom cell's 120^3 grid paired inside the
    adjoint chain's H applications (fused mode 2: the whole-plane kernel
    multiplies bwd(H^j y0)(r), formed just before its v(r) product, with the
    stored field bwd(g_j), g_j = sum_m c_{j+m+1} x_m) against the path that
    stores all eight real-space fields per state (fused mode 1); dL/da_k
    alike.  40 states: a full 32-state chunk and a last chunk of 8."""
    N = 2
    ak, G = laser(N)
    dstar = ad.target_dipole(N, scale=2e-3)
    cell, H, v, psi, occ = setup("c2", prec, natoms=8, nst=40)
    H.set_chunk(32)
    res = {}
    for fused in (1, 2):
        H.set_transform_config(0, 1, fused, 1)
        res[fused] = _grads(H, psi, occ, ak, G, N, 1, dstar)
    assert abs(res[2][0] - res[1][0]) < tol * abs(res[1][0])
    assert rel_err(res[2][1], res[1][1]) < tol
    assert rel_err(res[2][2], res[1][2]) < tol
