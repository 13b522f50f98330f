"""Dipole accuracy of the precision forms against the plain FP64 form.

    python -m qball_gb300.accuracy --config c2 --nst 32 --steps 200 [--hxc on|off]

Propagates the same delta-kicked state with each precision form through the
C ABI and records the total electronic current J(t) after every ETRS step
(CurrentDensity::update_current, CurrentDensity.cc:39-106, G-space form).
The dipole is d(t) = integral_0^t J dt' (trapezoid, FP64).  Reported per
form: max_t |d(t) - d64(t)| / max_t |d64(t)| for the kick direction and for
the vector norm, and the final relative wavefunction difference.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


# form label -> (precision form, projector GEMMs of the plain FP64 form)
FORMS = {"fp64": ("fp64", "ozaki"), "fp64_simt": ("fp64", "simt")}


def run_form(label, cell, basis, psi0, occ, A, dt, steps, chunk=0, hxc=True):
    import torch
    import qball_gb300 as Q
    from qball_gb300 import synth
    precision, gemm = FORMS.get(label, (label, None))
    H = Q.Hamiltonian(basis, *cell.grid, precision=precision)
    if gemm:
        H.set_fp64_gemm(gemm)
    if chunk:
        H.set_chunk(chunk)
    H.set_vlocal(synth.vlocal(cell))
    H.set_nonlocal(synth.species(cell))
    H.set_vector_potential(A)
    if hxc:
        synth.enable_selfconsistent(H, cell, psi0, occ)
    p = psi0.clone()
    nel = float(occ.sum())
    J = [H.current(p, occ, nel)]
    t0 = time.perf_counter()
    for _ in range(steps):
        H.etrs_step(p, occ, dt, A_t=A, A_tdt=A)
        J.append(H.current(p, occ, nel))
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    J = np.array(J)
    d = np.zeros_like(J)
    for k in range(1, len(J)):
        d[k] = d[k - 1] + 0.5 * dt * (J[k - 1] + J[k])
    H.close()
    return dict(J=J, d=d, psi=p, seconds=el)


def main():
    import torch
    import qball_gb300 as Q
    from qball_gb300 import synth
    sys.path.insert(0, os.path.dirname(HERE))

    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c2")
    ap.add_argument("--nst", type=int, default=0)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--dt", type=float, default=0.05)
    ap.add_argument("--forms", default="fp64,mixed")
    ap.add_argument("--out", default="")
    ap.add_argument("--ref", default="", help="npz of an earlier run: reuse its fp64 d(t)")
    ap.add_argument("--hxc", default="on", choices=["on", "off"],
                    help="self-consistent Hartree + LDA potential (as bench.py)")
    ap.add_argument("--simt-steps", type=int, default=0,
                    help="also run the FP64 form with FP64-FMA projector GEMMs for this many "
                         "steps and compare it with the tensor-core FP64 form over them")
    ap.add_argument("--json", default="", help="write the report to this file")
    args = ap.parse_args()
    kw = {"nst": args.nst} if args.nst else {}
    cell = synth.make_cell(args.config, **kw)
    basis = Q.Basis(cell.L, cell.ecut)
    psi0 = synth.device_wavefunctions(cell, basis)
    occ = synth.occupations(cell)
    A = synth.kick()
    res = {}
    for form in args.forms.split(","):
        res[form] = run_form(form, cell, basis, psi0, occ, A, args.dt, args.steps,
                             hxc=args.hxc == "on")
    if args.ref:
        z = np.load(args.ref)
        ref = {"d": z["fp64_d"][:args.steps + 1], "J": z["fp64_J"][:args.steps + 1], "psi": None}
        res.setdefault("fp64", ref)
    ref = res["fp64"]
    dref = ref["d"]
    scale_z = np.abs(dref[:, 2]).max()
    scale_n = np.linalg.norm(dref, axis=1).max()
    report = {"config": args.config, "nst": cell.nst, "steps": args.steps, "dt": args.dt,
              "hxc": args.hxc,
              "kick": list(A), "d64_final": list(map(float, dref[-1])), "forms": {}}
    for form, r in res.items():
        dd = r["d"] - dref
        rel_z = float(np.abs(dd[:, 2]).max() / scale_z)
        rel_n = float(np.linalg.norm(dd, axis=1).max() / scale_n)
        pd = (float(((r["psi"] - ref["psi"]).abs().pow(2).sum().sqrt()
                     / ref["psi"].abs().pow(2).sum().sqrt()).item())
              if r["psi"] is not None and ref["psi"] is not None else None)
        report["forms"][form] = {"dipole_rel_err_z": rel_z, "dipole_rel_err_norm": rel_n,
                                 "psi_rel_err_final": pd, "seconds": r.get("seconds"),
                                 "steps_per_s": (args.steps / r["seconds"]) if r.get("seconds")
                                 else None}
    if args.simt_steps > 0:
        # the FP64 trajectory itself against the FP64-FMA GEMMs over its first steps
        n = args.simt_steps
        r = run_form("fp64_simt", cell, basis, psi0, occ, A, args.dt, n, hxc=args.hxc == "on")
        r64 = run_form("fp64", cell, basis, psi0, occ, A, args.dt, n, hxc=args.hxc == "on")
        dn = r["d"][:n + 1]
        dz = np.abs(dn[:, 2]).max()
        report["fp64_vs_fp64_simt"] = {
            "steps": n,
            "dipole_rel_err_z": float(np.abs(r64["d"][:, 2] - dn[:, 2]).max() / dz),
            "current_max_abs_diff": float(np.abs(r64["J"] - r["J"]).max()),
            "psi_rel_err_final": float(((r64["psi"] - r["psi"]).abs().pow(2).sum().sqrt()
                                        / r["psi"].abs().pow(2).sum().sqrt()).item()),
            "seconds_per_step_simt": r["seconds"] / n}
    print(json.dumps(report), flush=True)
    if args.json:
        with open(args.json, "w") as f:
            json.dump(report, f, indent=1)
    if args.out:
        np.savez(args.out, **{f"{k}_d": v["d"] for k, v in res.items()},
                 **{f"{k}_J": v["J"] for k, v in res.items()})


if __name__ == "__main__":
    main()
