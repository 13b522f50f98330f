"""Multi-process (world size 2, gloo, CPU) cover of the state-sharded path.

The H|psi> / ETRS path is independent per state: the only exchange when
states are sharded over ranks is one sum of rho(r) per density build plus
scalar sums (electron count, current), the reference's
Context::dsum('r', ...) at ChargeDensity.cc:309 and CurrentDensity.cc:86-92.
Each rank here builds the density and current of its contiguous block of
states with the CPU oracle; the all-reduced sums must equal the one-rank
result.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import sys
    import torch
    import torch.distributed as dist
    root = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
    sys.path.insert(0, root)
    from oracle import oracle as O
    from qball_gb300 import synth
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cell = synth.make_cell("t12")
    b = O.Basis(np.diag([cell.L] * 3).reshape(9), cell.ecut)
    ft = O.FT(b, *cell.grid)
    psi = synth.wavefunctions(cell, b)
    occ = synth.occupations(cell)
    n0 = cell.nst * rank // world
    n1 = cell.nst * (rank + 1) // world
    rho, nel = O.update_density(ft, psi[n0:n1].T, occ[n0:n1])
    A = synth.kick()
    J = O.current_g(b, psi[n0:n1].T, occ[n0:n1], np.zeros(3), 0.0)
    t = torch.from_numpy(np.concatenate([rho, [nel], J]))
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    if rank == 0:
        out.put(t.numpy().copy())
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_state_sharded_density_and_current_sum():
    import sys
    root = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
    sys.path.insert(0, root)
    from oracle import oracle as O
    from qball_gb300 import synth
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = q.get(timeout=100)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    cell = synth.make_cell("t12")
    b = O.Basis(np.diag([cell.L] * 3).reshape(9), cell.ecut)
    ft = O.FT(b, *cell.grid)
    psi = synth.wavefunctions(cell, b)
    occ = synth.occupations(cell)
    rho, nel = O.update_density(ft, psi.T, occ)
    J = O.current_g(b, psi.T, occ, np.zeros(3), 0.0)
    n = ft.n012
    assert np.abs(res[:n] - rho).max() <= 1e-12 * np.abs(rho).max()
    assert abs(res[n] - nel) <= 1e-12 * nel
    assert np.abs(res[n + 1:] - J).max() <= 1e-12 * max(1.0, np.abs(J).max())


class _OracleOp:
    """The oracle adjoint behind the operator-pair interface of
    qball_gb300.TDPropagation (forward -> J, backward -> dL/da_n, grad_v)."""

    def __init__(self, td):
        self.td = td

    def forward(self, psi, A):
        self.A = A
        self.states, J = self.td.forward(psi, A)
        return J

    def backward(self, dLdJ, e=None, grad_v=None):
        gv, ga, _ = self.td.backward(self.states, self.A, dLdJ, e)
        if grad_v is not None:
            grad_v[:] = gv
        return ga


def _adjoint_problem(nst, n0, n1):
    from oracle import oracle as O
    from oracle.adjoint import TDAdjoint
    from qball_gb300 import adjoint as ad
    from qball_gb300 import synth
    cell = synth.make_cell("t12")
    b = O.Basis(np.diag([cell.L] * 3).reshape(9), cell.ecut)
    ft = O.FT(b, *cell.grid)
    psi = synth.wavefunctions(cell, b, nst=nst)
    occ = synth.occupations(cell, nst=nst)
    N, dt = 2, 0.05
    times = dt * np.arange(N + 1)
    tk, ak, sigma = ad.pulse_train(3, times[-1], seed=21, amp=0.05)
    G = ad.pulse_integrals(times, tk, sigma)
    e = np.array([0.0, 0.0, 1.0])
    A = ad.vector_potential(ak, G, e, A0=synth.kick())
    op = _OracleOp(TDAdjoint(b, ft, synth.vlocal(cell), synth.species(cell), occ[n0:n1], dt))
    gv = np.zeros(ft.n012)
    L, J, ga = ad.dipole_loss_gradients(op, np.asfortranarray(psi[n0:n1].T), A, dt,
                                        ad.target_dipole(N, scale=2e-3), e, grad_v=gv)
    return L, J, ga, gv


def _adjoint_worker(rank, world, port, out):
    import sys
    import torch.distributed as dist
    root = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
    sys.path.insert(0, root)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    nst = 4
    L, J, ga, gv = _adjoint_problem(nst, nst * rank // world, nst * (rank + 1) // world)
    if rank == 0:
        out.put((L, J, ga, gv))
    dist.destroy_process_group()


@pytest.mark.timeout(180)
def test_state_sharded_adjoint_gradients():
    """States split over 2 gloo ranks: the currents summed before the loss and
    the gradients summed after the backward pass equal the one-rank run."""
    import sys
    root = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
    sys.path.insert(0, root)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_adjoint_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    L2, J2, ga2, gv2 = q.get(timeout=150)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    L1, J1, ga1, gv1 = _adjoint_problem(4, 0, 4)
    assert abs(L2 - L1) <= 1e-12 * abs(L1)
    assert np.abs(J2 - J1).max() <= 1e-12 * np.abs(J1).max()
    assert np.abs(ga2 - ga1).max() <= 1e-10 * np.abs(ga1).max()
    assert np.abs(gv2 - gv1).max() <= 1e-10 * np.abs(gv1).max()
