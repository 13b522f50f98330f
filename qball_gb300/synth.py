"""Seeded synthetic cells for the H|psi> / ETRS path.

No public dataset is involved: every input is generated from a seed.
  * cubic cell of edge L (bohr), full-sphere basis at ecut (Ha);
  * atoms uniform in the cell, minimum separation 3 bohr (rejection);
  * psi(G) = complex normal * exp(-|G|^2/8), Gram/Cholesky-orthonormalised in
    FP64 (the semantics of SlaterDet::gram, SlaterDet.cc:1043-1143);
  * v_loc(r) = sum_a -2 exp(-|r - tau_a|^2 / (2 w^2)), w = 1 bohr, minimum
    image (the real-space form of a Gaussian local pseudopotential);
  * one KB species, lmax 1 (s,p: 4 projectors/atom) or 2 (s,p,d: 9/atom),
    radial form g^l exp(-g^2 rc^2/2) with rc = 1, weights D_l ~ U[0.5, 2] Ha;
  * occupations 2 (closed shell);
  * for the Hartree + xc update: the density basis of the largest cutoff
    (4 ecut at most) whose grid, by the reference's rule (ChargeDensity.cc:
    76-100), fits the cell's grid; vion_local_g the Fourier coefficients of
    the same Gaussian wells; rhopst Gaussian pseudo-charges -Z exp(-G^2
    rc^2/4)/Omega per atom (rc = 1 bohr), Z = electrons per atom, so that the
    cell is neutral.
"""
import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Cell:
    L: float
    ecut: float            # Hartree
    grid: tuple
    nst: int
    natoms: int
    lmax: int
    seed: int = 1234
    name: str = ""
    tau: np.ndarray = field(default=None, repr=False)
    wt: list = field(default=None, repr=False)


# the workloads of the benchmark configurations
CONFIGS = {
    # 8 atoms, L=20, 20 Ry, 48^3, 16 states, s+p projectors
    "c1": dict(L=20.0, ecut=10.0, grid=(48, 48, 48), nst=16, natoms=8, lmax=1),
    # 8 atoms on the reference's own dense-grid rule for this cell (64^3)
    "c1q": dict(L=20.0, ecut=10.0, grid=(64, 64, 64), nst=16, natoms=8, lmax=1),
    # 216 atoms, L=30, 50 Ry, 120^3, 432 states, s+p+d projectors
    "c2": dict(L=30.0, ecut=25.0, grid=(120, 120, 120), nst=432, natoms=216, lmax=2),
    # 512 atoms, L=40, 40 Ry, 160^3, 2048 states
    "c5": dict(L=40.0, ecut=20.0, grid=(160, 160, 160), nst=2048, natoms=512, lmax=2),
    # small cells for tests
    "t12": dict(L=12.0, ecut=10.0, grid=(32, 32, 32), nst=8, natoms=4, lmax=2),
    "t12b": dict(L=12.0, ecut=10.0, grid=(20, 24, 30), nst=5, natoms=3, lmax=2),
}


def make_cell(name=None, seed=1234, **kw):
    params = dict(CONFIGS[name]) if name else {}
    params.update(kw)
    c = Cell(seed=seed, name=name or "custom", **params)
    rng = np.random.default_rng(seed)
    c.tau = place_atoms(rng, c.L, c.natoms)
    c.wt = list(rng.uniform(0.5, 2.0, size=3))
    return c


def place_atoms(rng, L, n, min_sep=3.0, max_tries=200000):
    pts = []
    tries = 0
    while len(pts) < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError(f"could not place {n} atoms with separation {min_sep} in L={L}")
        p = rng.uniform(0.0, L, size=3)
        ok = True
        for q in pts:
            d = p - q
            d -= L * np.round(d / L)
            if np.dot(d, d) < min_sep * min_sep:
                ok = False
                break
        if ok:
            pts.append(p)
    return np.array(pts, dtype=np.float64).reshape(n, 3)


def species(cell):
    return [dict(tau=cell.tau, lmax=cell.lmax, rc=1.0, wt=cell.wt)]


def vlocal(cell, depth=-2.0, width=1.0):
    """v(r) on the grid, x fastest: index i + n0*(j + n1*k)."""
    n0, n1, n2 = cell.grid
    L = cell.L
    x = np.arange(n0) * (L / n0)
    y = np.arange(n1) * (L / n1)
    z = np.arange(n2) * (L / n2)
    v = np.zeros((n2, n1, n0))
    for t in cell.tau:
        def g1(r, c):
            d = r - c
            d -= L * np.round(d / L)
            return np.exp(-d * d / (2 * width * width))
        gx, gy, gz = g1(x, t[0]), g1(y, t[1]), g1(z, t[2])
        v += depth * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
    return v.reshape(-1)


def wavefunctions(cell, basis, seed=None, nst=None):
    """[nst, ngw] complex128, orthonormal rows."""
    rng = np.random.default_rng(cell.seed + 7 if seed is None else seed)
    n = cell.nst if nst is None else nst
    ngw = basis.ngw
    env = np.exp(-basis.kpg2 / 8.0)
    c = (rng.standard_normal((n, ngw)) + 1j * rng.standard_normal((n, ngw))) * env[None, :]
    return gram(c)


def gram(c):
    """Cholesky orthonormalisation of the rows of c (FP64)."""
    s = c.conj() @ c.T          # s_ij = <psi_i|psi_j>
    l = np.linalg.cholesky(s)   # s = L L^H
    # rows c' = conj(L)^{-1} c give <psi'_i|psi'_j> = delta_ij
    return np.linalg.solve(l.conj(), c)


def occupations(cell, nst=None):
    return np.full(cell.nst if nst is None else nst, 2.0)


def kick(strength=0.01):
    """velocity-gauge delta kick along z (set vector_potential 0 0 A)."""
    return np.array([0.0, 0.0, strength])


def _good(n):
    """Basis::factorizable (Basis.cc:126-150)."""
    for p in (11, 7, 5, 3, 3):
        if n % p == 0:
            n //= p
    while n % 2 == 0:
        n //= 2
    return n == 1


def rule_grid(L, ecut):
    """Edge of the cubic density grid the reference builds for cutoff ecut
    (Ha): vbasis np + 2, rounded up to a good size (ChargeDensity.cc:76-100,
    Basis.cc:560-573)."""
    hmax = int(0.5 + math.sqrt(2.0 * ecut) / (2.0 * math.pi) * L)
    n = 2 * hmax + 2
    while not _good(n):
        n += 2
    n += 2
    while not _good(n):
        n += 2
    return n


def density_ecut(cell):
    """Density cutoff (Ha): 4 ecut when the reference's grid for it fits the
    cell's grid, else the largest cutoff below that (0.25 Ha steps) that does
    (the ecutden option, ChargeDensity.cc:78-79)."""
    e = 4.0 * cell.ecut
    while e > cell.ecut and rule_grid(cell.L, e) > min(cell.grid):
        e -= 0.25
    return e


def ionic_terms(cell, vbasis, depth=-2.0, width=1.0, rcps=1.0, zv=None):
    """(vion_local_g, rhopst) [ngv] complex on the density basis.

    vion: coefficients of sum_a depth exp(-|r-tau_a|^2/(2 width^2)) (the wells
    of vlocal()), (2 pi width^2)^(3/2) depth exp(-G^2 width^2/2) S(G)/Omega;
    rhopst: -zv exp(-G^2 rcps^2/4) S(G)/Omega; S(G) = sum_a exp(-i G.tau_a).
    """
    g = vbasis.kpgx.reshape(3, -1)
    g2 = vbasis.kpg2
    if zv is None:
        zv = 2.0 * cell.nst / max(cell.natoms, 1)
    S = np.zeros(vbasis.ngw, np.complex128)
    for t in cell.tau:
        S += np.exp(-1j * (g[0] * t[0] + g[1] * t[1] + g[2] * t[2]))
    om = vbasis.omega
    vion = depth * (2.0 * np.pi * width * width) ** 1.5 * np.exp(-0.5 * g2 * width * width) * S / om
    rhopst = -zv * np.exp(-0.25 * g2 * rcps * rcps) * S / om
    return vion, rhopst


def enable_selfconsistent(H, cell, p, occ):
    """Density basis, ionic terms and v_r of the density of the device
    states p on the Hamiltonian H, then the self-consistent step
    (EhrenSampleStepper.cc:322-329 before the first step).  Returns the
    density basis."""
    import torch
    import qball_gb300 as Q
    vb = Q.Basis(cell.L, density_ecut(cell))
    vion, rhopst = ionic_terms(cell, vb)
    H.set_density_basis(vb)
    H.set_ionic_terms(vion, rhopst)
    rho = torch.empty(H.n012, dtype=torch.float64, device=p.device)
    H.update_density(p, occ, rho)
    H.update_vhxc(rho)
    H.set_selfconsistent(True)
    del rho
    return vb


def device_wavefunctions(cell, basis, nst=None):
    """Seeded random states on cuda, Gram-orthonormalised in FP64 by the
    library's SlaterDet::gram (qbg_gram: products on the device, the nst x nst
    Cholesky factor on the host); torch complex128 [nst, ngw]."""
    import torch
    import qball_gb300 as Q
    rng = np.random.default_rng(cell.seed + 7)
    n, ngw = (cell.nst if nst is None else nst), basis.ngw
    env = torch.from_numpy(np.exp(-basis.kpg2 / 8.0)).cuda()
    c = torch.empty((n, ngw), dtype=torch.complex128, device="cuda")
    for s0 in range(0, n, 64):
        s1 = min(n, s0 + 64)
        blk = rng.standard_normal((s1 - s0, ngw)) + 1j * rng.standard_normal((s1 - s0, ngw))
        c[s0:s1] = torch.from_numpy(blk).cuda() * env
    Q.FourierTransform(basis, *cell.grid).gram(c)
    return c
