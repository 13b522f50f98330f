"""Wavefunction checkpoints in the reference's "states" format.

Wavefunction::write_states / read_states (Wavefunction.cc:2406-2580,
2790-2970), binary format, one process row: one file per state and k-point
named

    <base>k<kp:04d>n<n:05d>            (one spin)
    <base>s<spin:1d>k<kp:04d>n<n:05d>  (two spins)

holding psi_n(r) = backward(c_n) on the basis' own grid (Basis::np) as
complex<double> values in grid order (x fastest), with no header; reading
transforms each file forward (with 1/N) back to the coefficients.  With
empty states the reference also writes <base>[s<spin>]k<kp:04d>.occ holding
eig[nst] then occ[nst] (doubles).  Files are written and read in the host's
byte order, as the reference does.

The transforms are the caller's: `device_transforms(basis)` gives the
product's (the C ABI's qbg_backward / qbg_forward on a plan of the basis'
grid, FP64); any pair of callables with the same meaning works.
"""
import os

import numpy as np


def state_file(base, n, kp=0, spin=None):
    """File name of state n of k-point kp (spin None: one spin)."""
    if spin is None:
        return f"{base}k{kp:04d}n{n:05d}"
    return f"{base}s{spin:1d}k{kp:04d}n{n:05d}"


def occ_file(base, kp=0, spin=None):
    if spin is None:
        return f"{base}k{kp:04d}.occ"
    return f"{base}s{spin:1d}k{kp:04d}.occ"


def write_states(base, c, backward, kp=0, spin=None, eig=None, occ=None):
    """Write the states c ([nst, ngw] host array) through backward(c_n) ->
    psi(r) (complex128, N values); eig and occ (both or neither) go to the
    .occ file.  Returns the list of state files."""
    c = np.asarray(c)
    names = []
    for n in range(c.shape[0]):
        f = np.ascontiguousarray(backward(c[n]), dtype=np.complex128)
        name = state_file(base, n, kp, spin)
        with open(name, "wb") as fh:
            fh.write(f.tobytes())
        names.append(name)
    if (eig is None) != (occ is None):
        raise ValueError("write_states: give both eig and occ, or neither")
    if eig is not None:
        e = np.ascontiguousarray(eig, np.float64)
        o = np.ascontiguousarray(occ, np.float64)
        if e.shape != (c.shape[0],) or o.shape != (c.shape[0],):
            raise ValueError("write_states: eig and occ need one value per state")
        with open(occ_file(base, kp, spin), "wb") as fh:
            fh.write(e.tobytes())
            fh.write(o.tobytes())
    return names


def read_states(base, nst, n012, forward, kp=0, spin=None, with_occ=False):
    """Read nst states of n012 grid points each and transform them with
    forward(psi(r)) -> c_n.  Returns c [nst, ngw] (and (eig, occ) when
    with_occ).  A missing or short file raises (the reference aborts)."""
    out = []
    for n in range(nst):
        name = state_file(base, n, kp, spin)
        if not os.path.exists(name):
            raise FileNotFoundError(f"{name}: checkpoint file not found")
        f = np.fromfile(name, dtype=np.complex128)
        if f.size < n012:
            raise ValueError(f"{name}: {f.size} values, the grid has {n012}")
        out.append(np.asarray(forward(f[:n012])))
    c = np.stack(out)
    if not with_occ:
        return c
    eo = np.fromfile(occ_file(base, kp, spin), dtype=np.float64)
    if eo.size < 2 * nst:
        raise ValueError(f"{occ_file(base, kp, spin)}: {eo.size} values, expected {2 * nst}")
    return c, eo[:nst].copy(), eo[nst:2 * nst].copy()


def device_transforms(basis):
    """(backward, forward) of one state through a plan on the basis' own grid
    (FP64), on host arrays: each call copies to the device, transforms with
    qbg_backward / qbg_forward and copies back."""
    import torch
    import qball_gb300 as Q
    ft = Q.FourierTransform(basis, *basis.np)
    N = int(np.prod(basis.np))

    def backward(cn):
        c = torch.from_numpy(np.ascontiguousarray(cn, np.complex128).reshape(1, -1)).cuda()
        f = torch.zeros((1, N), dtype=torch.complex128, device="cuda")
        ft.backward(c, f)
        return f.cpu().numpy()[0]

    def forward(fr):
        f = torch.from_numpy(np.array(fr, np.complex128).reshape(1, -1)).cuda()
        c = torch.zeros((1, basis.ngw), dtype=torch.complex128, device="cuda")
        ft.forward(f, c)
        return c.cpu().numpy()[0]

    backward.plan = forward.plan = ft
    return backward, forward
