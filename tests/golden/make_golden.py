"""Generate the golden vectors in tests/golden/ from the reference itself.

Runs the reference's own Basis::resize and FourierTransform::backward /
forward (serial FFT_NOLIB build) and LDAFunctional::setxc, compiled from the
reference sources into oracle/_ref by oracle/build_ref.sh, on seeded inputs
and stores the results.
The reference's tests pin nothing on this path, so these files are the pins
for the oracle restatement (oracle/qbo.c) and for the product's basis
builder.  Usage:

    export QBG_REFERENCE=<reference tree>
    sh oracle/build_ref.sh && python tests/golden/make_golden.py [name ...]

(names: the CASES below, "lda" and "species"; all when none is given).
"species" reads two pseudopotentials of the reference's test suite with the
reference's own Species code and stores their projector tables.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from oracle import oracle as O  # noqa: E402

# (name, L bohr, ecut Ha, FFT grid or None)
CASES = [
    ("l12_e10", 12.0, 10.0, (20, 24, 30)),
    ("l12_e10_g32", 12.0, 10.0, (32, 32, 32)),
    ("l20_e10_g48", 20.0, 10.0, (48, 48, 48)),
    ("l20_e10_g64", 20.0, 10.0, (64, 64, 64)),
    ("l30_e25", 30.0, 25.0, None),
    ("l40_e20", 40.0, 20.0, None),
]


def weight_field(grid):
    """Smooth real weight w(r) = 1 + 0.5 cos(...) on the grid (x fastest)."""
    n0, n1, n2 = grid
    k, j, i = np.meshgrid(np.arange(n2), np.arange(n1), np.arange(n0), indexing="ij")
    return (1.0 + 0.5 * np.cos(2 * np.pi * (i / n0 + 2 * j / n1 + 3 * k / n2))).reshape(-1)


def case_inputs(b, seed=20260):
    rng = np.random.default_rng(seed)
    env = np.exp(-b.kpg2 / 8)
    c1 = (rng.standard_normal(b.ngw) + 1j * rng.standard_normal(b.ngw)) * env
    c2 = (rng.standard_normal(b.ngw) + 1j * rng.standard_normal(b.ngw)) * env
    return c1, c2


def lda_densities():
    """Densities spanning both branches of the correlation fit (rs < 1 and
    rs >= 1, rs = 1 at rho = 3/(4 pi)), zero and negative values."""
    rng = np.random.default_rng(11)
    rs1 = 3.0 / (4.0 * np.pi)
    return np.concatenate([
        [0.0, -1e-3, -1.0, 1e-300],
        np.logspace(-14, 4, 361),
        rs1 * (1.0 + np.linspace(-1e-6, 1e-6, 21)),
        rng.uniform(0.0, 0.2, 200),
    ])


def make_lda():
    rho = lda_densities()
    exc, vxc = O.ref_lda(rho)
    np.savez_compressed(os.path.join(HERE, "ref_lda.npz"), rho=rho, exc=exc, vxc=vxc)
    print("lda", rho.size)


# Species of the reference's own test suite (paths relative to its
# testsuite/pseudopotentials folder), read and initialised by the reference's
# Species code: ONCV xenon (UPF, s/p/d, two channels) and argon (QSO XML,
# s/p, two channels).
SPECIES = [("Xe", "02_xenon_upf/Xe_ONCV_PBE-1.1.upf", 2),
           ("Ar", "07_argon_oncv/Ar_ONCV_PBE-1.1.xml", 2)]
SPECIES_CELL = dict(L=12.0, ecut=10.0, grid=(32, 32, 32), A=(0.0, 0.0, 0.01), seed=31)


def species_tables(h, info, kpgxA, kpg2A):
    """twnl[ipr][ig], lproj[ipr], wt[ipr] of one species as
    NonLocalPotential::init and update_twnl build them for Kleinman-Bylander
    projectors (nquad = 0; NonLocalPotential.cc:205-250 and the l = 0, 1, 2
    branches of :306-760): for each l != llocal and each channel ic, the 2l+1
    real harmonics at k+G-A times the radial projector Species::dvnlg(l, ic,
    |k+G-A|) of the reference's own Species; weights Species::wsg(l, ic)."""
    lmax, lloc, nch = int(info[0]), int(info[1]), int(info[2])
    fpi = 4.0 * np.pi
    s14pi, s34pi, s54pi, s3 = np.sqrt(1 / fpi), np.sqrt(3 / fpi), np.sqrt(5 / fpi), np.sqrt(3.0)
    tg = np.sqrt(kpg2A)
    tgi = np.where(kpg2A > 0, 1.0 / np.where(kpg2A > 0, tg, 1.0), 0.0)
    tgx, tgy, tgz = kpgxA
    rows, lproj, wt = [], [], []
    for l in range(lmax + 1):
        if l == lloc:
            continue
        if l > 2:
            raise SystemExit("species with f projectors are not used here")
        for ic in range(nch):
            v = O.ref_species_vnlg(h, l, ic, tg)
            if l == 0:
                ys = [s14pi * np.ones_like(tg)]
            elif l == 1:
                ys = [s34pi * tgx * tgi, s34pi * tgy * tgi, s34pi * tgz * tgi]
            else:
                tgi2 = tgi * tgi
                xx, yy, zz = tgx * tgx * tgi2, tgy * tgy * tgi2, tgz * tgz * tgi2
                ys = [s54pi * 0.5 * (3.0 * zz - 1.0), s54pi * 0.5 * s3 * (xx - yy),
                      s54pi * s3 * (tgx * tgy * tgi2), s54pi * s3 * (tgy * tgz * tgi2),
                      s54pi * s3 * (tgx * tgz * tgi2)]
            w = O.ref_species_wsg(h, l, ic)
            for y in ys:
                rows.append(y * v)
                lproj.append(l)
                wt.append(w)
    return np.array(rows), np.array(lproj, np.int32), np.array(wt)


def make_species(root):
    """Projector tables of two testsuite species on a small cell, from the
    reference's own pseudopotential readers and Species::initialize."""
    c = SPECIES_CELL
    a = np.diag([c["L"]] * 3).reshape(9)
    b = O.Basis(a, c["ecut"], use_ref=True)
    A = np.array(c["A"])
    g = b.kpgx.reshape(3, -1)
    kpgxA = g - A[:, None]
    kpg2A = (g * g).sum(0) + A @ A - 2 * (A @ g)
    rng = np.random.default_rng(c["seed"])
    out = dict(a=a, ecut=np.float64(c["ecut"]), grid=np.array(c["grid"]), A=A,
               names=np.array([n for n, _, _ in SPECIES]),
               files=np.array([f for _, f, _ in SPECIES]))
    taus = rng.uniform(0.0, c["L"], size=(sum(n for _, _, n in SPECIES), 3))
    k = 0
    for i, (name, rel, na) in enumerate(SPECIES):
        h = O.ref_species_load(os.path.join(root, "testsuite", "pseudopotentials", rel), 1.0)
        info = O.ref_species_info(h)
        twnl, lproj, wt = species_tables(h, info, kpgxA, kpg2A)
        out[f"twnl{i}"] = twnl
        out[f"lproj{i}"] = lproj
        out[f"wt{i}"] = wt
        out[f"tau{i}"] = taus[k:k + na]
        out[f"info{i}"] = info
        # radial projectors on a |G| grid, for checks of the tables
        gg = np.linspace(0.0, 12.0, 97)
        out[f"vnlg_g{i}"] = gg
        out[f"vnlg{i}"] = np.array([[O.ref_species_vnlg(h, l, ic, gg) for ic in range(info[2])]
                                    for l in range(info[0] + 1)])
        O.ref_species_destroy(h)
        k += na
        print(name, rel, "lmax/llocal/nch/nlm", info[:4], "npr", len(lproj))
    path = os.path.join(HERE, "ref_species_xe_ar.npz")
    np.savez_compressed(path, **out)
    print("species", b.ngw, os.path.getsize(path))


def main(names=None):
    if O.ref() is None:
        raise SystemExit("oracle/_ref/libqbref.so is not built (run oracle/build_ref.sh)")
    if not names or "lda" in names:
        make_lda()
    if not names or "species" in names:
        root = os.environ.get("QBG_REFERENCE")
        if not root:
            raise SystemExit("QBG_REFERENCE must name the reference tree for the species tables")
        make_species(root)
    for name, L, ecut, grid in CASES:
        if names and name not in names:
            continue
        a = np.diag([L, L, L]).reshape(9)
        b = O.Basis(a, ecut, use_ref=True)
        out = dict(a=a, ecut=np.float64(ecut), ngw=b.ngw, nrods=b.nrods,
                   np=np.array(b.np), idxmin=np.array(b.idxmin), idxmax=np.array(b.idxmax),
                   rod_h=b.rod_h, rod_k=b.rod_k, rod_lmin=b.rod_lmin, rod_size=b.rod_size)
        rng = np.random.default_rng(7)
        sel = np.sort(rng.choice(b.ngw, size=min(b.ngw, 2048), replace=False))
        out["g_sel"] = sel
        out["kpg2_sel"] = b.kpg2[sel]
        out["kpgx_sel"] = b.kpgx.reshape(3, -1)[:, sel]
        if grid is not None:
            ft = O.RefFT(a, ecut, *grid)
            c1, c2 = case_inputs(b)
            f1 = ft.backward(c1)
            # rs_mul_add-shaped forward input: w(r) * backward(c2)
            r = ft.backward(c2) * weight_field(grid)
            cr = ft.forward(r)
            fsel = np.sort(rng.choice(ft.n012, size=min(ft.n012, 4096), replace=False))
            out.update(grid=np.array(grid), c1=c1, c2=c2, f_sel=fsel, f1_sel=f1[fsel],
                       f1_norm2=np.float64(np.vdot(f1, f1).real), c_from_r=cr,
                       c1_roundtrip=ft.forward(f1))
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **out)
        print(name, b.ngw, b.nrods, b.np, os.path.getsize(os.path.join(HERE, f"ref_{name}.npz")))


if __name__ == "__main__":
    main(sys.argv[1:])
