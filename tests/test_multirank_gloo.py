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
