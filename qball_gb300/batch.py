"""Many independent cells propagated together (the batched workload).

    python -m qball_gb300.batch [--cells 64] [--steps 4] [--form mixed_df32]

Seeded cells: edge L in [12, 24] bohr, cutoff 20-40 Ry, 4-64 atoms (s, p
projectors), 8-256 states, each on one of the 32/48/64/96-point cubic grids
that hold its basis (drawn at random).  Every cell gets its own plan, psi and
vector-potential kick, and is stepped (a) one cell after another through
qbg_etrs_step and (b) as one CUDA graph holding one ETRS step of every cell
as concurrent branches (qbg_etrs_graph_*).  Before timing, each plan picks
its states-per-launch-group with qbg_plan_autotune.  Prints one JSON line:
aggregate cell-steps/s of both ways and the largest relative difference
between their states.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

GRIDS = (32, 48, 64, 96)


def batch_cells(n, seed):
    """(L, ecut Ha, grid, natoms, nst) for n seeded cells."""
    import qball_gb300 as Q
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        L = float(rng.uniform(12.0, 24.0))
        ecut = float(rng.uniform(20.0, 40.0)) / 2.0
        nst = int(rng.integers(8, 257))
        natoms = int(min(rng.integers(4, 65), 0.3 * (L / 3.0) ** 3))
        b = Q.Basis(L, ecut)
        fit = [g for g in GRIDS if g >= max(b.np)]
        if not fit:
            continue
        out.append((L, ecut, int(fit[rng.integers(0, len(fit))]), natoms, nst))
    return out


def _shape_counts(cfgs):
    """How many plans the autotuner put on each transform shape."""
    out = {}
    for c in cfgs:
        k = (f"order{c['radix_order']}-pfa{c['prime_factor']}-fused{c['fused']}-"
             f"lane{c['lane_group']}-chunk{c['chunk']}")
        out[k] = out.get(k, 0) + 1
    return dict(sorted(out.items()))


def main():
    import torch
    import qball_gb300 as Q
    from qball_gb300 import synth
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=64)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--form", default="mixed_df32")
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--dt", type=float, default=0.05)
    ap.add_argument("--compare", default="",
                    help="comma-separated forms whose per-cell error after --compare-steps "
                         "ETRS steps is measured against the FP64 form (e.g. mixed,mixed_df32)")
    ap.add_argument("--compare-steps", type=int, default=2)
    args = ap.parse_args()
    torch.cuda.set_device(0)
    specs = batch_cells(args.cells, args.seed)
    A = synth.kick()
    seq, bat = [], []
    t0 = time.perf_counter()
    for i, (L, ecut, g, natoms, nst) in enumerate(specs):
        cell = synth.make_cell(None, seed=args.seed * 1000 + i, L=L, ecut=ecut, grid=(g, g, g),
                               nst=nst, natoms=natoms, lmax=1)
        b = Q.Basis(cell.L, cell.ecut)
        psi = torch.from_numpy(synth.wavefunctions(cell, b)).cuda()
        occ = synth.occupations(cell)
        for dst in (seq, bat):
            H = Q.Hamiltonian(b, *cell.grid, precision=args.form)
            H.set_vlocal(synth.vlocal(cell))
            H.set_nonlocal(synth.species(cell))
            H.set_vector_potential(A)
            dst.append((H, psi.clone(), occ))
    for H, p, occ in seq + bat:
        H.autotune(p, occ)
    setup_s = time.perf_counter() - t0
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            for H, p, occ in seq:
                H.etrs_step(p, occ, args.dt, stream=stream)
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            for H, p, occ in seq:
                H.etrs_step(p, occ, args.dt, stream=stream)
        e1.record(stream)
        stream.synchronize()
        ms_seq = e0.elapsed_time(e1)
    # device time of one step of every cell with each kernel run alone (the
    # plan's per-phase profiler): what the graph would take with no launch
    # cost and no overlap between cells
    busy_ms = 0.0
    clones = [p.clone() for _, p, _ in seq]
    torch.cuda.synchronize()
    for (H, _, occ), q in zip(seq, clones):
        H.profile(True)
        H.etrs_step(q, occ, args.dt, stream=stream)
        busy_ms += sum(v[0] for v in H.profile_read().values())
        H.profile(False)
    stream.synchronize()
    launches_per_step = 0
    for (H, _, occ), q in zip(seq, clones):
        l0 = H.launches()
        H.etrs_step(q, occ, args.dt, stream=stream)
        launches_per_step += H.launches() - l0
    stream.synchronize()
    del clones
    graph = Q.EtrsGraph(bat, args.dt, stream=stream)
    for _ in range(args.warmup):
        graph.launch(stream=stream)
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        graph.launch(stream=stream)
    e1.record(stream)
    stream.synchronize()
    graph.check()
    ms_graph = e0.elapsed_time(e1)
    diff = 0.0
    for (_, ps, _), (_, pb, _) in zip(seq, bat):
        d = (ps - pb).abs().pow(2).sum().sqrt() / ps.abs().pow(2).sum().sqrt()
        diff = max(diff, float(d))
    n = len(specs)
    line = {
        "workload": f"{n} seeded cells: L 12-24 bohr, 20-40 Ry, grids {list(GRIDS)}, 4-64 atoms "
                    f"(s,p projectors), 8-256 states, delta kick, form {args.form}",
        "cells": n, "states_total": int(sum(s[4] for s in specs)),
        "grids": {str(g): sum(1 for s in specs if s[2] == g) for g in GRIDS},
        "steps": args.steps, "warmup": args.warmup,
        "cell_steps_per_s_graph": n * args.steps / (ms_graph / 1000.0),
        "cell_steps_per_s_sequential": n * args.steps / (ms_seq / 1000.0),
        "graph_speedup": ms_seq / ms_graph,
        "ms_per_step_graph": ms_graph / args.steps,
        "kernel_device_ms_per_step": busy_ms,
        "kernel_launches_per_step": launches_per_step,
        "max_rel_diff_graph_vs_sequential": diff,
        "chunks": sorted({H.chunk for H, _, _ in bat}),
        "transform_shapes": _shape_counts([H.transform_config() for H, _, _ in bat]),
        "setup_s": setup_s,
        "device_gb_in_use": (lambda f: (f[1] - f[0]) / 1e9)(torch.cuda.mem_get_info()),
    }
    if args.compare:
        del seq, bat, graph
        torch.cuda.empty_cache()
        line["per_cell_error"] = compare_forms(specs, args)
    print(json.dumps(line), flush=True)


def compare_forms(specs, args):
    """Per cell: relative error of psi and of the current J after a few ETRS
    steps of each reduced form against the FP64 form (complex128 storage and
    arithmetic, tensor-core FP64-accurate projector GEMMs) on the same cell,
    one cell at a time."""
    import torch
    import qball_gb300 as Q
    from qball_gb300 import synth
    forms = [f for f in args.compare.split(",") if f]
    A = synth.kick()
    rows = []
    for i, (L, ecut, g, natoms, nst) in enumerate(specs):
        cell = synth.make_cell(None, seed=args.seed * 1000 + i, L=L, ecut=ecut, grid=(g, g, g),
                               nst=nst, natoms=natoms, lmax=1)
        b = Q.Basis(cell.L, cell.ecut)
        psi0 = torch.from_numpy(synth.wavefunctions(cell, b)).cuda()
        occ = synth.occupations(cell)
        out = {}
        for form in ["fp64"] + forms:
            H = Q.Hamiltonian(b, *cell.grid, precision=form)
            H.set_vlocal(synth.vlocal(cell))
            H.set_nonlocal(synth.species(cell))
            H.set_vector_potential(A)
            p = psi0.clone()
            for _ in range(args.compare_steps):
                H.etrs_step(p, occ, args.dt)
            out[form] = (p, H.current(p, occ, float(occ.sum())))
            H.close()
        p64, J64 = out["fp64"]
        row = {"grid": g, "nst": nst, "natoms": natoms}
        for form in forms:
            p, J = out[form]
            row[form] = {"psi": float(((p - p64).abs().pow(2).sum().sqrt()
                                       / p64.abs().pow(2).sum().sqrt()).item()),
                         "J": float(np.abs(J - J64).max() / max(np.abs(J64).max(), 1e-300))}
        rows.append(row)
        del out, psi0
        torch.cuda.empty_cache()
    summary = {f: {"psi_max": max(r[f]["psi"] for r in rows),
                   "psi_median": float(np.median([r[f]["psi"] for r in rows])),
                   "J_max": max(r[f]["J"] for r in rows)} for f in forms}
    return {"steps": args.compare_steps, "reference": "fp64 form", "summary": summary,
            "cells": rows}


if __name__ == "__main__":
    main()
