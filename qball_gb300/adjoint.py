"""Dipole-loss gradients through the checkpointed adjoint of the ETRS step.

    python -m qball_gb300.adjoint --config c2 --steps 20 --K 10 [--form mixed_df32]

Host side of the differentiation workload: a laser pulse train
E(t) = sum_k a_k exp(-(t - t_k)^2 / 2 sigma^2) along e enters the velocity
gauge as A' = -E (VectorPotential.h:150-160), so
    A(t_n) = A_0 - e sum_k a_k G_k(t_n),
    G_k(t) = int_0^t exp(-(s - t_k)^2 / 2 sigma^2) ds
           = sigma sqrt(pi/2) [erf((t - t_k)/(sigma sqrt 2)) + erf(t_k/(sigma sqrt 2))].
The dipole is d(t_n) = int_0^{t_n} J dt (trapezoid over the step currents)
and the loss L = sum_n (d_z(t_n) - d*_z(t_n))^2 against a target dipole
from a seeded random walk.  The device part (qbg_td_forward/backward) gives
dL/dJ -> dL/dv(r) and dL/da_n; this module maps dL/d(dipole) to dL/dJ and
dL/da_n to dL/da_k.  The CLI times one forward pass and one backward pass on
a seeded cell and prints one JSON line.
"""
import argparse
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def pulse_train(nk, t_end, seed=11, sigma=0.5, amp=0.02):
    """Seeded centres t_k in [0, t_end] and amplitudes a_k (a.u.)."""
    rng = np.random.default_rng(seed)
    tk = np.sort(rng.uniform(0.0, t_end, nk))
    ak = amp * rng.standard_normal(nk)
    return tk, ak, sigma


def pulse_integrals(times, tk, sigma):
    """G[n, k] = int_0^{t_n} exp(-(s - t_k)^2 / 2 sigma^2) ds."""
    s2 = sigma * math.sqrt(2.0)
    c = sigma * math.sqrt(math.pi / 2.0)
    erf = np.vectorize(math.erf)
    return c * (erf((times[:, None] - tk[None, :]) / s2) + erf(tk[None, :] / s2))


def vector_potential(ak, G, e, A0=(0.0, 0.0, 0.0)):
    """A[n] = A0 - e sum_k a_k G[n, k]; dA[n]/da_k = -e G[n, k]."""
    a = -(G @ ak)
    return np.asarray(A0, float)[None, :] + a[:, None] * np.asarray(e, float)[None, :]


def dipole(J, dt):
    """d[n] = trapezoid integral of J up to t_n (d[0] = 0)."""
    d = np.zeros_like(J)
    for n in range(1, len(J)):
        d[n] = d[n - 1] + 0.5 * dt * (J[n - 1] + J[n])
    return d


def target_dipole(nsteps, seed=5, scale=1e-3):
    """Seeded random walk d*_z(t_n)."""
    rng = np.random.default_rng(seed)
    return np.concatenate([[0.0], np.cumsum(scale * rng.standard_normal(nsteps))])


def loss_and_dJ(J, dt, dstar):
    """L = sum_n (d_z[n] - d*[n])^2 and dL/dJ[n] (shape of J)."""
    d = dipole(J, dt)
    r = d[:, 2] - dstar
    L = float(np.sum(r * r))
    gd = 2.0 * r  # dL/dd_z[n]
    # d[n] = dt/2 (J_0 + 2 J_1 + ... + 2 J_{n-1} + J_n)
    N = len(J) - 1
    suffix = np.concatenate([np.cumsum(gd[::-1])[::-1], [0.0]])  # suffix[m] = sum_{n>=m} gd[n]
    gJ = np.zeros_like(J)
    for m in range(N + 1):
        if m == 0:
            gJ[m, 2] = 0.5 * dt * suffix[1]
        else:
            gJ[m, 2] = 0.5 * dt * gd[m] + dt * suffix[m + 1]
    return L, gJ


def grad_amplitudes(grad_a, G):
    """dL/da_k = sum_n dL/da_n dA_n/da_k along e = -sum_n grad_a[n] G[n, k]."""
    return -(G.T @ grad_a)


def _sum_over_ranks(x):
    """In-place sum over the ranks of the default process group of a numpy
    array or torch tensor (host arrays travel through the device under NCCL)."""
    import torch
    import torch.distributed as dist
    if torch.is_tensor(x):
        dist.all_reduce(x)
        return x
    t = torch.from_numpy(x)
    if dist.get_backend() == "nccl":
        d = t.cuda()
        dist.all_reduce(d)
        t.copy_(d.cpu())
    else:
        dist.all_reduce(t)
    return x


def dipole_loss_gradients(op, psi, A, dt, dstar, e, grad_v=None):
    """One forward and backward pass of the dipole loss through the operator
    pair op (TDPropagation: forward(psi, A) -> J, backward(dLdJ, e, grad_v)
    -> dL/da_n).  When a process group of several ranks is initialised, each
    rank holds a block of the states: the step currents are summed over the
    ranks before the loss (J is a sum over states, the reference's
    Context::dsum at CurrentDensity.cc:86-92), and dL/dv(r) and dL/da_n after
    the backward pass (sums over states).  Returns (L, J, dL/da_n)."""
    import torch.distributed as dist
    sharded = dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1
    J = op.forward(psi, A)
    if sharded:
        _sum_over_ranks(J)
    L, gJ = loss_and_dJ(J, dt, dstar)
    ga = op.backward(gJ, e=e, grad_v=grad_v)
    if sharded:
        _sum_over_ranks(ga)
        if grad_v is not None:
            _sum_over_ranks(grad_v)
    return L, J, ga


def main():
    sys.path.insert(0, os.path.dirname(HERE))
    import torch
    import qball_gb300 as Q
    from qball_gb300 import synth
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c2")
    ap.add_argument("--form", default="mixed_df32")
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--K", type=int, default=10)
    ap.add_argument("--nst", type=int, default=0)
    ap.add_argument("--dt", type=float, default=0.05)
    ap.add_argument("--pulses", type=int, default=64)
    args = ap.parse_args()
    torch.cuda.set_device(0)
    kw = {"nst": args.nst} if args.nst else {}
    cell = synth.make_cell(args.config, **kw)
    b = Q.Basis(cell.L, cell.ecut)
    H = Q.Hamiltonian(b, *cell.grid, precision=args.form)
    H.set_vlocal(synth.vlocal(cell))
    H.set_nonlocal(synth.species(cell))
    psi0 = synth.device_wavefunctions(cell, b)
    occ = synth.occupations(cell)
    N, dt = args.steps, args.dt
    times = dt * np.arange(N + 1)
    tk, ak, sigma = pulse_train(args.pulses, times[-1])
    G = pulse_integrals(times, tk, sigma)
    e = np.array([0.0, 0.0, 1.0])
    A = vector_potential(ak, G, e, A0=synth.kick())
    dstar = target_dipole(N)
    td = Q.TDPropagation(H, psi0, occ, dt, N, K=args.K)
    grad_v = torch.zeros(H.n012, dtype=torch.float64, device="cuda:0")
    # warm-up: one step each way on a one-step operator (tables, work buffers)
    w = Q.TDPropagation(H, psi0, occ, dt, 1, K=1)
    p = psi0.clone()
    w.forward(p, A[:2])
    w.backward(np.zeros((2, 3)), e=e, grad_v=grad_v)
    w.close()
    torch.cuda.synchronize()
    p = psi0.clone()
    t0 = time.perf_counter()
    J = td.forward(p, A)
    t1 = time.perf_counter()
    L, gJ = loss_and_dJ(J, dt, dstar)
    t2 = time.perf_counter()
    ga = td.backward(gJ, e=e, grad_v=grad_v)
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    gk = grad_amplitudes(ga, G)
    fwd_ms = (t1 - t0) * 1e3 / N
    bwd_ms = (t3 - t2) * 1e3 / N
    gv = grad_v.cpu().numpy()
    print(json.dumps({
        "workload": f"{cell.natoms} atoms, {cell.grid[0]}^3, {psi0.shape[0]} states, {N} laser-driven "
                    f"ETRS steps (dt {dt}), {args.pulses} Gaussian pulses (sigma {sigma}) along z, "
                    f"dipole loss, checkpoint every {args.K} steps, form {args.form}",
        "forward_ms_per_step": fwd_ms, "backward_ms_per_step": bwd_ms,
        "backward_over_forward": bwd_ms / fwd_ms,
        "loss": L, "grad_v_norm": float(np.linalg.norm(gv)),
        "grad_amplitudes_norm": float(np.linalg.norm(gk)),
        "device_gb_in_use": (lambda f: (f[1] - f[0]) / 1e9)(torch.cuda.mem_get_info()),
    }), flush=True)
    td.close()


if __name__ == "__main__":
    main()
