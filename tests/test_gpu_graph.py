"""Batched cells stepped as one CUDA graph, and the chunk autotuner.

A graph replay must give the same states as stepping every cell on its own
(same kernels in the same order per cell: bitwise, checked to 1e-13), for
cells of different grids, forms and state counts, with and without the
self-consistent potential; the autotuner must keep H|psi> unchanged.
"""
import numpy as np
import pytest

from conftest import rel_err
import qball_gb300 as Q
from qball_gb300 import synth

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


def dev(x):
    return _torch().from_numpy(np.ascontiguousarray(x)).to("cuda:0")


def make(name, prec, hxc=False, **kw):
    cell = synth.make_cell(name, **kw)
    b = Q.Basis(cell.L, cell.ecut)
    H = Q.Hamiltonian(b, *cell.grid, precision=prec)
    H.set_vlocal(synth.vlocal(cell))
    H.set_nonlocal(synth.species(cell))
    H.set_vector_potential(synth.kick())
    psi = synth.wavefunctions(cell, b)
    occ = synth.occupations(cell)
    if hxc:
        vb = Q.Basis(cell.L, synth.density_ecut(cell))
        H.set_density_basis(vb)
        vion, rhopst = synth.ionic_terms(cell, vb)
        H.set_ionic_terms(vion, rhopst)
        torch = _torch()
        rho = torch.zeros(H.n012, dtype=torch.float64, device="cuda:0")
        H.update_density(dev(psi), occ, rho)
        H.update_vhxc(rho)
        H.set_selfconsistent(True)
    return H, psi, occ


CELLS = [("t12", "fp64", False, {}), ("t12b", "mixed_df32", False, {}),
         ("c1", "mixed_df32", False, {"nst": 8}), ("t12", "mixed", True, {"grid": (40, 40, 40)})]


def test_graph_replay_matches_individual_steps(cuda):
    torch = _torch()
    ref, bat = [], []
    for name, prec, hxc, kw in CELLS:
        H1, psi, occ = make(name, prec, hxc, **kw)
        H2, _, _ = make(name, prec, hxc, **kw)
        ref.append((H1, dev(psi), occ))
        bat.append((H2, dev(psi), occ))
    dt = 0.05
    stream = torch.cuda.Stream()
    g = Q.EtrsGraph(bat, dt, stream=stream)
    for _ in range(2):
        g.launch(stream=stream)
    g.check()
    for H, p, occ in ref:
        for _ in range(2):
            H.etrs_step(p, occ, dt)
    torch.cuda.synchronize()
    for (_, pr, _), (_, pb, _) in zip(ref, bat):
        assert rel_err(pb.cpu().numpy(), pr.cpu().numpy()) < 1e-13
    g.close()


def test_graph_cells_match_the_oracle(cuda):
    """Two batched cells of different grids (FP64 form, fixed potential)
    after two graph replays against the oracle's ETRS steps of each cell."""
    from oracle import oracle as O
    torch = _torch()
    cells = []
    for name in ("t12", "t12b"):
        H, psi, occ = make(name, "fp64")
        cells.append((name, H, dev(psi), occ, psi))
    stream = torch.cuda.Stream()
    g = Q.EtrsGraph([(H, p, occ) for _, H, p, occ, _ in cells], 0.05, stream=stream)
    for _ in range(2):
        g.launch(stream=stream)
    g.check()
    for name, H, p, occ, psi in cells:
        cell = synth.make_cell(name)
        oh = O.Ham(O.FT(O.Basis(H.basis.a, cell.ecut), *cell.grid), synth.vlocal(cell),
                   synth.species(cell))
        A = synth.kick()
        oh.set_A(A)
        ref = psi.T.copy()
        for _ in range(2):
            ref, _, _ = oh.etrs_step(ref, occ, 0.05, A, A, nthreads=8)
        assert rel_err(p.cpu().numpy(), ref.T) < 1e-10, name
    g.close()


def test_graph_rejects_repeated_plan(cuda):
    H, psi, occ = make("t12", "fp64")
    p = dev(psi)
    with pytest.raises(Q.QbgError, match="repeats"):
        Q.EtrsGraph([(H, p, occ), (H, p, occ)], 0.05)


def test_autotune_keeps_hpsi(cuda):
    torch = _torch()
    H, psi, occ = make("c1", "mixed_df32")
    p = dev(psi)
    before = torch.zeros_like(p)
    H.hpsi(p, before, occ)
    ch = H.autotune(p, occ)
    assert ch in (8, 16, 32, 64)
    cfg = H.transform_config()
    assert cfg["chunk"] == ch and cfg["radix_order"] in (0, 1, 2)
    after = torch.zeros_like(p)
    H.hpsi(p, after, occ)
    assert rel_err(after.cpu().numpy(), before.cpu().numpy()) < 1e-12


@pytest.mark.parametrize("name,prec,tol", [("t12", "fp64", 1e-13), ("c1", "fp64", 1e-13),
                                           ("c1", "mixed_df32", 1e-11), ("c1", "mixed", 1e-5)])
def test_every_transform_shape_gives_the_same_hpsi(cuda, name, prec, tol):
    """Every transform shape the autotuner can pick (radix order of the
    Stockham passes, prime-factor splits, fused x-y-x kernel, register
    lane-group y pass) gives the same H|psi> to the rounding of the form."""
    torch = _torch()
    H, psi, occ = make(name, prec)
    p = dev(psi)
    ref = torch.zeros_like(p)
    H.hpsi(p, ref, occ)
    r = ref.cpu().numpy()
    seen = 0
    for order in (0, 1, 2):
        for pfa in (1, 0):
            for fused in (1, 0):
                for lane in (1, 0):
                    if fused and not pfa:
                        continue
                    H.set_transform_config(order, pfa, fused, lane)
                    assert H.transform_config()["radix_order"] == order
                    out = torch.zeros_like(p)
                    H.hpsi(p, out, occ)
                    assert rel_err(out.cpu().numpy(), r) < tol, (order, pfa, fused, lane)
                    seen += 1
    assert seen == 18


def test_bounded_wait_expires_and_context_survives(cuda):
    """A device wait on a barrier that nothing completes gives up after its
    poll limit with QBG_ERR_TIMEOUT (no hang, no fault); the GPU keeps
    working afterwards."""
    assert Q.selftest_wait_timeout(20000) == 5  # QBG_ERR_TIMEOUT
    assert "bounded wait expired" in Q.lib().qbg_last_error().decode()
    torch = _torch()
    H, psi, occ = make("t12", "fp64")
    out = torch.zeros_like(dev(psi))
    H.hpsi(dev(psi), out, occ)
    torch.cuda.synchronize()
    assert torch.isfinite(out.abs()).all()


@pytest.mark.parametrize("prec", ["mixed_df32", "mixed", "fp64"])
def test_gemm_wait_expiry_reported_by_the_same_call(cuda, prec):
    """Every pipeline wait of the tensor-core GEMMs made to give up at once
    (poll limit 0) on a non-blocking stream: the ETRS step that ran the
    GEMMs returns QBG_ERR_TIMEOUT itself (the error word is read on the
    caller's stream), each CTA drains its own copies and MMAs before it frees
    its memory, and the plan is usable again afterwards."""
    torch = _torch()
    H, psi, occ = make("t12", prec)
    p = dev(psi)
    ref = torch.zeros_like(p)
    H.hpsi(p, ref, occ)
    s = torch.cuda.Stream()  # non-blocking with respect to the legacy stream
    H.set_wait_polls(0)
    with pytest.raises(Q.QbgError, match="timeout"):
        H.etrs_step(p.clone(), occ, 0.05, stream=s)
    with pytest.raises(Q.QbgError, match="timeout"):
        H.hpsi(p, torch.zeros_like(p), occ, stream=s)
    H.set_wait_polls(-1)
    out = torch.zeros_like(p)
    H.hpsi(p, out, occ, stream=s)
    s.synchronize()
    assert rel_err(out.cpu().numpy(), ref.cpu().numpy()) < 1e-14
