"""Profiling driver: ETRS steps or H|psi> applications of a synthetic cell.

    python -m qball_gb300.profile_step --form mixed_df32 --nst 432 --steps 1
    python -m qball_gb300.profile_step --form mixed_df32 --natoms 8 --nst 16 --hpsi 3

Meant to run under ncu: it builds the same workload as bench.py (seeded cell,
normalised random states; no torch.linalg call, which does not load under
ncu) and runs either full ETRS steps or bare H|psi> applications.  --natoms
shrinks the projector set (and its multi-GB tables) while keeping the grid,
basis and states -- the transform kernels then do exactly the work they do in
the benchmark.
"""
import argparse
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def main():
    import torch
    import qball_gb300 as Q
    from qball_gb300 import synth
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c2")
    ap.add_argument("--form", default="mixed_df32")
    ap.add_argument("--nst", type=int, default=0)
    ap.add_argument("--natoms", type=int, default=0)
    ap.add_argument("--steps", type=int, default=0)
    ap.add_argument("--hpsi", type=int, default=0)
    ap.add_argument("--hxc", default="on", choices=["on", "off"],
                    help="self-consistent Hartree + LDA potential in the ETRS steps")
    ap.add_argument("--phases", action="store_true",
                    help="after one warm-up H|psi>, time the --hpsi applications with the "
                         "library's per-phase profiler (each launch alone) and print the mean "
                         "ms per H of every phase as JSON; not for use under ncu")
    args = ap.parse_args()
    kw = {}
    if args.nst:
        kw["nst"] = args.nst
    if args.natoms:
        kw["natoms"] = args.natoms
    cell = synth.make_cell(args.config, **kw)
    b = Q.Basis(cell.L, cell.ecut)
    H = Q.Hamiltonian(b, *cell.grid, precision=args.form)
    H.set_vlocal(synth.vlocal(cell))
    H.set_nonlocal(synth.species(cell))
    rng = np.random.default_rng(1)
    env = torch.from_numpy(np.exp(-b.kpg2 / 8)).cuda()
    psi = torch.empty((cell.nst, b.ngw), dtype=torch.complex128, device="cuda")
    for s0 in range(0, cell.nst, 64):
        s1 = min(cell.nst, s0 + 64)
        blk = rng.standard_normal((s1 - s0, b.ngw)) + 1j * rng.standard_normal((s1 - s0, b.ngw))
        psi[s0:s1] = torch.from_numpy(blk).cuda() * env
    psi /= psi.abs().pow(2).sum(dim=1, keepdim=True).sqrt()
    occ = np.full(cell.nst, 2.0)
    A = synth.kick()
    H.set_vector_potential(A)
    if args.hxc == "on":
            synth.enable_selfconsistent(H, cell, psi, occ)
    out = torch.zeros_like(psi)
    if args.phases and args.hpsi:
        H.hpsi(psi, out, occ)
        H.profile(True)
    for _ in range(args.hpsi):
        H.hpsi(psi, out, occ)
    if args.phases and args.hpsi:
        pr = H.profile_read()
        H.profile(False)
        import json
        print(json.dumps({"form": args.form, "natoms": cell.natoms, "nst": cell.nst,
                          "ms_per_H": {k: round(v[0] / args.hpsi, 3)
                                       for k, v in pr.items() if v[1]}}))
    for _ in range(args.steps):
        H.etrs_step(psi, occ, 0.05, A_t=A, A_tdt=A)
    torch.cuda.synchronize()
    print("ok", args.form, cell.nst, cell.natoms, H.launches())


if __name__ == "__main__":
    main()
