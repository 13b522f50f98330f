#!/usr/bin/env python3
"""ETRS steps/s on the 216-atom cell: mixed precision vs the plain FP64 form.

`value` times the precision form given by --form (default mixed_df32:
double-float transforms on the FP32 pipe, projector GEMMs on the tensor
cores) -- the fastest form whose 200-step dipole stays within 1e-8 (relative)
of the plain FP64 form (profiles/accuracy.json, produced by python -m
qball_gb300.accuracy).  The FP32-transform form, the FP64-transform form and
the plain FP64 form are timed beside it under `other_forms`.

One "step" is one ETRS step of EhrenSampleStepper with the
ExponentialWavefunctionStepper (preupdate + update: three 4th-order Taylor
exponentials = 12 H|psi> applications) over all 432 states of the synthetic
216-atom cell (L = 30 bohr, ecut 50 Ry, 120^3 grid, 161 235 full-sphere
plane waves, 9 KB projectors per atom), delta-kicked by A = (0, 0, 0.01),
with the self-consistent Hamiltonian (--hxc on, the default): the density of
psi(t) and of the predicted psi(t+dt) each rebuild v_r = v_ion + v_H + v_xc
(LDA) on the 135 Ry density sphere that the 120^3 grid holds.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` is whole-job ETRS steps/s of the
mixed form with psi resident in HBM (psi is 1.1 GB, far larger than L2, so
no flush is needed between steps); `e2e` is the same step through the
public API with psi copied in from pinned host memory and psi(t+dt) plus
the current J read back every step (the copies run on a second stream and
overlap the neighbouring steps).  `fp64_gpu` times the plain FP64 form
on the same cell.  With N > 1 each rank propagates its own replica (no
data-path collective; weak scaling).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "TDDFT ETRS steps/s (216 at.) mixed vs FP64 GPU at <=1e-8 dipole rel err"


def workload_config(cfg, cell, ngw, ngv, dt, hxc):
    """The `config` object of both arms: the workload and its Hamiltonian."""
    return {"workload": f"{cfg}: {cell.natoms} atoms, L={cell.L:g} bohr, ecut {2 * cell.ecut:g} Ry, "
                        f"grid {cell.grid[0]}^3, {ngw} PW (full sphere), {cell.nst} states, "
                        f"{nproj_of(cell)} KB projectors, ETRS dt={dt}, delta kick A_z=0.01",
            "hamiltonian": (f"self-consistent: v_ion + Hartree + LDA rebuilt from the density of "
                            f"psi(t) and of the predicted psi(t+dt) every step, density sphere "
                            f"{2 * synth_density_ecut(cell):g} Ry ({ngv} G)" if hxc else
                            "fixed local potential")}


def synth_density_ecut(cell):
    from qball_gb300 import synth
    return synth.density_ecut(cell)


def metric_for(cell):
    """The metric's name with the atom count of the cell actually timed."""
    return METRIC.replace("(216 at.)", f"({cell.natoms} at.)")
UNIT = "steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2")
    ap.add_argument("--dt", type=float, default=0.05)
    ap.add_argument("--fp64-steps", type=int, default=1)
    ap.add_argument("--fp64-warmup", type=int, default=1)
    ap.add_argument("--e2e-steps", type=int, default=8)
    ap.add_argument("--e2e-warmup", type=int, default=2)
    ap.add_argument("--cpu-states", type=int, default=16)
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--aetrs-steps", type=int, default=3,
                    help="steps of the headline form with the AETRS propagator option "
                         "(0: not timed)")
    ap.add_argument("--fp64-slices", type=int, default=7, choices=[6, 7],
                    help="7-bit slices per operand of the FP64 form's tensor-core GEMMs")
    ap.add_argument("--fp64-simt-steps", type=int, default=0,
                    help="ETRS steps of the FP64 form with FP64-FMA projector GEMMs (0: one "
                         "profiled H|psi> only; a step takes ~40 s on the 216-atom cell)")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--chunk", type=int, default=0)
    ap.add_argument("--hxc", default="on", choices=["on", "off"],
                    help="self-consistent Hartree + LDA potential inside the step")
    ap.add_argument("--form", default="mixed_df32",
                    help="precision form timed for `value` (the fastest form whose 200-step "
                         "dipole error is within 1e-8 of the FP64 form)")
    ap.add_argument("--also", default="mixed,mixed_fft64",
                    help="comma-separated forms timed beside it")
    ap.add_argument("--also-steps", type=int, default=3)
    ap.add_argument("--also-warmup", type=int, default=3)
    return ap.parse_args()


# ------------------------------------------------------------ distributed
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------ clocks
class Clocks:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], None, set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
                power.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "power_w_median": float(np.median(power)) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ------------------------------------------------------------ system
def make_system(cfg, precision, psi_np=None, chunk=0):
    import qball_gb300 as Q
    from qball_gb300 import synth
    cell = synth.make_cell(cfg)
    basis = Q.Basis(cell.L, cell.ecut)
    H = Q.Hamiltonian(basis, *cell.grid, precision=precision)
    if chunk:
        H.set_chunk(chunk)
    H.set_vlocal(synth.vlocal(cell))
    H.set_nonlocal(synth.species(cell))
    if psi_np is None:
        psi_np = synth.device_wavefunctions(cell, basis)
    return cell, basis, H, psi_np


def time_etrs(H, p, occ, dt, A, steps, warmup, stream):
    import torch
    for _ in range(warmup):
        H.etrs_step(p, occ, dt, A_t=A, A_tdt=A, stream=stream)
    torch.cuda.synchronize()
    l0 = H.launches()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        H.etrs_step(p, occ, dt, A_t=A, A_tdt=A, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), H.launches() - l0


# ------------------------------------------------------------ roofline
# FP32-pipe instructions of one double-float line transform, counted by
# instantiating the codelets of qbg_fft_engine.cuh with an operation-counting
# scalar (double-float add 8 instructions, multiply 4, halving 2): 120 = 8 x 15
# prime-factor = 15 dft8 (432) + 8 dft15 (1500); 48 = 3 dft16 (1280) + 16 dft3
# (108).  Other lengths: the 120 ratio to the 5 n log2 n model.
DF32_INST_PER_LINE = {120: 18480.0, 48: 5568.0}


def _fft_flops(n):
    return 5.0 * n * np.log2(n)


def _df32_inst(n):
    return DF32_INST_PER_LINE.get(n, _fft_flops(n) * 18480.0 / _fft_flops(120))


def arith_peaks():
    """FP32 FFMA and FP64 DFMA peaks (TFLOP/s) measured on the GB300s
    (profiles/peaks_gb300.json)."""
    with open(os.path.join(HERE, "profiles", "peaks_gb300.json")) as f:
        pk = json.load(f)
    return float(pk["fp32_ffma_tflops"]), float(pk["fp64_dfma_tflops"])


def phase_model(H, cell, basis):
    """Algorithmic work per STATE of each timed phase: (amount, bound, peak).

    Transform phases count line transforms: for double-float forms the amount
    is 2 x the FP32-pipe instructions of the algorithm (FFMA-equivalent
    flops, against the FP32 FFMA peak); for FP64 and FP32 forms the 5 n log2 n
    flops of the reference's own FFT model (src/tests/testFourierTransform.cc)
    against the FP64 or FP32 peak.  GEMM phases count 2 M N K per real
    product (3 split products on the tensor pipe in the mixed forms)."""
    n0, n1, n2 = cell.grid
    ngw, nrods = basis.ngw, basis.nrods
    nband = 2 * (max(abs(basis.idxmin[1]), abs(basis.idxmax[1])) + 1)
    P = nproj_of(cell)
    prec = H.precision
    f32, f64 = arith_peaks()
    if prec == "mixed_df32":
        w, fb = (lambda n: 2.0 * _df32_inst(n)), ("fp32", f32)
    elif prec in ("fp64", "mixed_fft64"):
        w, fb = _fft_flops, ("fp64", f64)
    else:
        w, fb = _fft_flops, ("fp32", f32)
    tc = prec in ("mixed", "mixed_fft64", "mixed_df32")
    # executed slice products per real GEMM on the tensor pipe: 3 (2-piece
    # FP16 split) in the mixed forms; Ozaki slices S in the FP64 form:
    # S (S + 1) / 2 pairs
    oz = prec == "fp64" and getattr(H, "fp64_gemm", "simt") == "ozaki"
    nprod = 3 if tc else (H.oz_slices * (H.oz_slices + 1) // 2 if oz else 1)
    lines = {
        "ft_z_bwd": nrods * w(n2),
        "ft_z_fwd": nrods * w(n2),
        "ft_x_bwd": n2 * nband * w(n0),
        "ft_x_fwd": n2 * nband * w(n0),
        "ft_y_vloc": n2 * n0 * 2 * w(n1),
        "ft_xyx_vloc": n2 * (2 * nband * w(n0) + 2 * n0 * w(n1)),
        "ft_y_density": n2 * (nband * w(n0) + n0 * w(n1)),
    }
    m = {k: (v, fb) for k, v in lines.items()}
    gemm = 8.0 * P * ngw  # one complex GEMM, per state
    m["fnl_gemm"] = (nprod * gemm, ("tensor", None) if (tc or oz) else ("fp64", f64))
    m["enl_hpsi"] = m["fnl_gemm"]
    return m


def nproj_of(cell):
    return cell.natoms * (cell.lmax + 1) ** 2


def phase_bytes(H, cell, basis):
    """Algorithmic HBM bytes per STATE of each transform phase of one H|psi>
    (the z-column intermediate in and out, psi in, H psi out, the v(r) tile
    once per launch group of H.chunk states)."""
    n0, n1, n2 = cell.grid
    ngw, nrods = basis.ngw, basis.nrods
    cs = 8 if H.precision in ("mixed", "mixed_nl64") else 16  # complex transform element
    vs = {"mixed_df32": 8, "mixed": 4, "mixed_nl64": 4}.get(H.precision, 8)
    zrows = cs * n2 * nrods
    N = n0 * n1 * n2
    return {"ft_z_bwd": 16 * ngw + zrows,
            "ft_z_fwd": zrows + 2 * 16 * ngw,
            "ft_xyx_vloc": 2 * zrows + N * vs / max(1, H.chunk),
            "ft_y_density": zrows + N * 8 / max(1, H.chunk)}


def roofline_of(H, cell, basis, prof, peaks, nst):
    """The dominant phase of one H application (largest device time), against
    the bound the roofline contract names: the tensor pipe for the GEMMs, HBM
    for everything else (with the compute pipe that actually bounds a
    transform beside it as compute_view)."""
    model = phase_model(H, cell, basis)
    dom = max((k for k in model if k in prof and prof[k][1]), key=lambda k: prof[k][0])
    tot_ms, nl = prof[dom]
    amount, (bound, peak) = model[dom]
    if bound == "tensor":
        peak = float(peaks.get("bf16_tflops", 1917.4))
    achieved = amount * nst / (tot_ms / 1000.0) / 1e12
    traffic = None
    try:
        tr = json.load(open(os.path.join(HERE, "profiles", "traffic.json")))
        key = f"{H.precision}:{dom}"
        if key in tr:
            traffic = tr[key]["bytes_per_launch"]
    except (OSError, ValueError):
        pass
    unit = ("TFLOP/s (FFMA-equivalent: 2 x FP32-pipe instructions of the double-float "
            "algorithm per second)" if H.precision == "mixed_df32" and dom.startswith("ft_")
            else "TFLOP/s")
    per_launch_ms = tot_ms / max(nl, 1)
    hbm_view = None
    if traffic:
        # the same launches against the measured HBM copy bandwidth: DRAM
        # bytes per launch (ncu) over the live per-launch time
        hbm_peak = float(peaks.get("hbm_gbs", 6785.5))
        hbm_gbs = traffic / (per_launch_ms / 1000.0) / 1e9
        hbm_view = {"bound": "hbm", "achieved": hbm_gbs, "peak": hbm_peak, "unit": "GB/s",
                    "frac": hbm_gbs / hbm_peak,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks
                    else "fallback 6785.5 GB/s"}
    compute = {"pipe": bound, "achieved": achieved, "peak": peak, "unit": unit,
               "frac": achieved / peak,
               "peak_source": ("MEASURED_PEAKS.json bf16_tflops (FP16 kind::f16 runs at the "
                               "same rate)" if bound == "tensor"
                               else "profiles/peaks_gb300.json")}
    if bound == "tensor":
        head = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "peak_source": compute["peak_source"]}
    else:
        # algorithmic bytes per launch over the live per-launch time
        hbm_peak = float(peaks.get("hbm_gbs", 6785.5))
        alg = phase_bytes(H, cell, basis).get(dom, 0.0) * nst / max(nl, 1)
        gbs = alg / (per_launch_ms / 1000.0) / 1e9
        head = {"bound": "hbm", "achieved": gbs, "peak": hbm_peak, "unit": "GB/s",
                "frac": gbs / hbm_peak, "algorithmic_bytes_per_launch": alg,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks
                else "fallback 6785.5 GB/s"}
    return {"kernel": dom, **head, "traffic": traffic, "compute_view": compute,
            "hbm_view_measured_traffic": hbm_view,
            "per_launch_ms": per_launch_ms, "launches_per_H": nl,
            "phases_ms_per_H": {k: round(v[0], 3) for k, v in prof.items() if v[1]},
            "phase_frac_of_peak": {k: round(model[k][0] * nst / (v[0] / 1000.0) / 1e12 /
                                            (float(peaks.get("bf16_tflops", 1917.4))
                                             if model[k][1][0] == "tensor" else model[k][1][1]), 4)
                                   for k, v in prof.items() if v[1] and k in model}}


# ------------------------------------------------------------ CPU baseline
def cpu_baseline(cfg, nsample, reps=1, hxc=True):
    """The CPU oracle (plain-C restatement of the reference path, OpenMP over
    states) on a bounded sample: H|psi> and the density of `nsample` states of
    the full cell; one ETRS step is extrapolated as 12 H + 2 densities over
    all states (both linear in the number of states) plus two Hartree + LDA
    updates of the potential on the full grid (with hxc; else 12 H + 1
    density)."""
    from oracle import oracle as O
    import qball_gb300 as Q
    from qball_gb300 import synth
    cell = synth.make_cell(cfg)
    b = O.Basis(Q.cubic_cell(cell.L), cell.ecut)
    ft = O.FT(b, *cell.grid)
    v = synth.vlocal(cell)
    ham = O.Ham(ft, v, synth.species(cell))
    ham.set_A(synth.kick())
    rng = np.random.default_rng(5)
    c = (rng.standard_normal((b.ngw, nsample)) + 1j * rng.standard_normal((b.ngw, nsample)))
    c = np.asfortranarray(c * np.exp(-b.kpg2 / 8)[:, None])
    occ = np.full(nsample, 2.0)
    cores = os.cpu_count() or 1
    th = []
    for _ in range(reps):
        t0 = time.perf_counter()
        ham.hpsi(c, occ, nthreads=cores)
        t1 = time.perf_counter()
        O.update_density(ft, c, occ, nthreads=cores)
        t2 = time.perf_counter()
        th.append((t1 - t0, t2 - t1))
    th = np.array(th)
    t_h, t_d = float(th[:, 0].min()), float(th[:, 1].min())
    scale = cell.nst / nsample
    t_v = 0.0
    if hxc:
        vb = O.Basis(Q.cubic_cell(cell.L), synth.density_ecut(cell))
        vion, rhopst = synth.ionic_terms(cell, vb)
        hx = O.Hxc(vb, *cell.grid, vion, rhopst)
        rho, _ = O.update_density(ft, c, occ, nthreads=cores)
        t0 = time.perf_counter()
        hx.update_vhxc(rho)
        t_v = time.perf_counter() - t0
    nd = 2 if hxc else 1
    step_s = (12 * t_h + nd * t_d) * scale + 2 * t_v
    extra = f" + 2 x Hartree/LDA update ({t_v:.2f} s, 1 thread)" if hxc else ""
    return {"value": 1.0 / step_s, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": (f"oracle H|psi> ({t_h:.2f} s) + density ({t_d:.2f} s) of {nsample} of "
                       f"{cell.nst} states of the full {cfg} cell, {cores} threads; ETRS step "
                       f"= (12 H + {nd} density) x {scale:.0f}{extra}")}


# ------------------------------------------------------------ arms
def run_reference(args, rank, world):
    if rank != 0:
        return
    K, W = max(1, args.steps), max(0, args.warmup)
    vals = []
    res = None
    for i in range(W + K):
        res = cpu_baseline(args.config, args.cpu_states, hxc=args.hxc == "on")
        if i >= W:
            vals.append(res["value"])
    v = float(np.median(vals))
    res["value"] = v
    from oracle import oracle as O
    import qball_gb300 as Q
    from qball_gb300 import synth
    cell = synth.make_cell(args.config)
    hxc = args.hxc == "on"
    ngw = O.Basis(Q.cubic_cell(cell.L), cell.ecut).ngw
    ngv = O.Basis(Q.cubic_cell(cell.L), synth.density_ecut(cell)).ngw if hxc else 0
    line = {"impl": "reference", "metric": metric_for(cell), "value": v, "unit": UNIT,
            "n_gpus": args.gpus, "steps": K, "warmup": W, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": workload_config(args.config, cell, ngw, ngv, args.dt, hxc),
            "cpu_baseline": res,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def accuracy_table(cfg):
    """Measured 200-step dipole errors of each form against the FP64 form for
    the cell `cfg` (profiles/accuracy.json, python -m qball_gb300.accuracy);
    {} when that cell was not measured."""
    try:
        a = json.load(open(os.path.join(HERE, "profiles", "accuracy.json")))
    except (OSError, ValueError):
        return {}
    ent = a.get("by_config", {}).get(cfg, {})
    return ent.get("forms", {})


def run_ours(args, rank, world, local):
    import torch
    from qball_gb300 import synth
    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    acc = accuracy_table(args.config)
    cell, basis, H, psi = make_system(args.config, args.form, chunk=args.chunk)
    occ = synth.occupations(cell)
    A = synth.kick()
    H.set_vector_potential(A)
    hxc = args.hxc == "on"
    vb = synth.enable_selfconsistent(H, cell, psi, occ) if hxc else None
    p = psi.clone()
    barrier(world)
    clocks = Clocks(local)
    clocks.start()
    ms, launches = time_etrs(H, p, occ, args.dt, A, args.steps, args.warmup, stream)
    clk = clocks.stop()
    barrier(world)
    ms_max = allreduce_max(ms, world)
    value = world * args.steps / (ms_max / 1000.0)

    # per-phase device time of one H application (profiled: launches run alone)
    hp = torch.empty_like(p)
    H.profile(True)
    H.hpsi(p, hp, occ, stream=stream)
    prof = H.profile_read()
    # and of one density of all states (the step builds two)
    rho_t = torch.empty(H.n012, dtype=torch.float64, device=p.device)
    H.profile(True)
    H.update_density(p, occ, rho_t, stream=stream)
    prof_rho = {k: round(v[0], 3) for k, v in H.profile_read().items() if v[1]}
    H.profile(False)
    del rho_t
    roofline = roofline_of(H, cell, basis, prof, peaks, cell.nst)
    roofline["phases_ms_per_density"] = prof_rho

    # end to end through the public API with host buffers: every step copies
    # its input psi in from pinned host memory and its result psi(t+dt) and J
    # back.  Two device buffers and a copy stream let step k+1's input and
    # step k-1's result move while step k computes (a serving pipeline); the
    # timed region spans the first copy in to the last copy out.
    e2e = None
    if not args.skip_e2e:
        nbytes = p.numel() * p.element_size()
        h_in = torch.empty(p.shape, dtype=p.dtype, pin_memory=True)
        h_in.copy_(psi)
        h_out = torch.empty_like(h_in, pin_memory=True)
        bufs = [p, torch.empty_like(p)]
        cs = torch.cuda.Stream()

        def e2e_run(nsteps):
            ev_in = [torch.cuda.Event(), torch.cuda.Event()]
            start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            start.record(stream)
            cs.wait_event(start)
            with torch.cuda.stream(cs):
                bufs[0].copy_(h_in, non_blocking=True)
                ev_in[0].record(cs)
            J = None
            for k in range(nsteps):
                if k + 1 < nsteps:
                    with torch.cuda.stream(cs):  # after the copy-out of step k-1
                        bufs[(k + 1) % 2].copy_(h_in, non_blocking=True)
                        ev_in[(k + 1) % 2].record(cs)
                b = bufs[k % 2]
                stream.wait_event(ev_in[k % 2])
                H.etrs_step(b, occ, args.dt, A_t=A, A_tdt=A, stream=stream)
                J = H.current(b, occ, float(occ.sum()), stream=stream)
                done = torch.cuda.Event()
                done.record(stream)
                cs.wait_event(done)
                with torch.cuda.stream(cs):
                    h_out.copy_(b, non_blocking=True)
            last = torch.cuda.Event()
            last.record(cs)
            stream.wait_event(last)
            end.record(stream)
            torch.cuda.synchronize()
            return start.elapsed_time(end), J

        if args.e2e_warmup:
            e2e_run(args.e2e_warmup)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ms, J = e2e_run(args.e2e_steps)
        wall = time.perf_counter() - t0
        e2e_ms = allreduce_max(ms, world)
        e2e = {"value": world * args.e2e_steps / (e2e_ms / 1000.0), "unit": UNIT,
               "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes + 24,
               "steps": args.e2e_steps, "warmup": args.e2e_warmup, "wall_s": wall,
               "pipeline": "copies on a second stream overlap the neighbouring steps",
               "J_last": list(map(float, J))}
        del bufs
        del h_in, h_out
    del H
    torch.cuda.empty_cache()

    # the other forms on the same cell and states
    others = {}
    # (label, form, FP64 GEMM, steps, warm-up); 0 steps: one profiled H|psi> only
    runs = [(f, f, None, args.also_steps, args.also_warmup) for f in args.also.split(",") if f]
    if args.aetrs_steps:
        # the same form with the stepper's AETRS option (a different
        # propagator: 8 H|psi> and one density per step once three
        # potentials are stored; the warm-up stores them)
        runs.append((args.form + "_aetrs", args.form, None, args.aetrs_steps, 3))
    if not args.skip_fp64:
        runs.append(("fp64", "fp64", "ozaki", args.fp64_steps, args.fp64_warmup))
        runs.append(("fp64_simt", "fp64", "simt", args.fp64_simt_steps, args.fp64_warmup
                     if args.fp64_simt_steps else 0))
    for label, form, gemm, steps, warm in runs:
        _, _, H2, _ = make_system(args.config, form, psi_np=psi)
        if gemm:
            H2.set_fp64_gemm(gemm, args.fp64_slices)
        H2.set_vector_potential(A)
        if hxc:
            synth.enable_selfconsistent(H2, cell, psi, occ)
        if label.endswith("_aetrs"):
            H2.set_aetrs(True)
        p2 = psi.clone()
        ent = {"unit": UNIT, "steps": steps, "warmup": warm,
               "dipole_rel_err_200_steps": acc.get(label)}
        if steps:
            ms2, _ = time_etrs(H2, p2, occ, args.dt, A, steps, warm, stream)
            ms2 = allreduce_max(ms2, world)
            ent["value"] = world * steps / (ms2 / 1000.0)
        H2.profile(True)
        H2.hpsi(p2, hp, occ, stream=stream)
        pr2 = H2.profile_read()
        H2.profile(False)
        ent["phases_ms_per_H"] = {k: round(v[0], 3) for k, v in pr2.items() if v[1]}
        # each phase against the pipe that bounds it in this form (FP64 pipe
        # for FP64 transforms, tensor pipe for the GEMMs)
        model2 = phase_model(H2, cell, basis)
        ent["phase_frac_of_peak"] = {
            k: round(model2[k][0] * cell.nst / (v[0] / 1000.0) / 1e12 /
                     (float(peaks.get("bf16_tflops", 1917.4)) if model2[k][1][0] == "tensor"
                      else model2[k][1][1]), 4)
            for k, v in pr2.items() if v[1] and k in model2}
        ent["phase_bound"] = {k: model2[k][1][0] for k, v in pr2.items() if v[1] and k in model2}
        others[label] = ent
        del H2, p2
        torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        cpu = cpu_baseline(args.config, args.cpu_states, hxc=hxc)

    if rank == 0:
        form_desc = {
            "mixed_df32": "double-float (FP32 pair) transforms, tensor-core projector GEMMs "
                          "(FP16 2-piece split, compensated accumulation), FP64 kinetic/Taylor/"
                          "reductions",
            "mixed_fft64": "FP64 transforms, tensor-core projector GEMMs (FP16 2-piece split, "
                           "FP32 accumulate per 256, compensated), FP64 kinetic/Taylor/reductions",
            "mixed": "FP32 transforms, tensor-core projector GEMMs (FP16 2-piece split), FP64 "
                     "kinetic/Taylor/reductions",
            "fp64": "FP64 throughout; projector GEMMs FP64-accurate on the tensor cores "
                    "(Ozaki scheme: 7 slices of 7 bits, exact FP32 windows)",
            "fp64_simt": "FP64 throughout; projector GEMMs as FP64 FMAs on the CUDA cores"}
        line = {"metric": metric_for(cell), "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64 + f16-split tensor GEMM" if args.form != "fp64" else "f64",
                "form": args.form, "form_desc": form_desc.get(args.form, args.form),
                "dipole_rel_err_200_steps": acc.get(args.form),
                "data": "synthetic (seeded cell, random orthonormal states)",
                "config": {**workload_config(args.config, cell, basis.ngw,
                                             vb.ngw if hxc else 0, args.dt, hxc),
                           "l2": f"inputs (psi {psi.numel() * 16 / 1e9:.1f} GB) larger than L2; "
                                 "no flush",
                           "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
                "gpu_launches": launches, "clocks": clk, "roofline": roofline,
                "e2e": e2e, "other_forms": others, "cpu_baseline": cpu}
        if "value" in others.get("fp64", {}):
            line["speedup_vs_fp64_gpu"] = value / others["fp64"]["value"]
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
