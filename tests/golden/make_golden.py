"""Generate the golden vectors in tests/golden/ from the reference itself.

Runs the reference's own Basis::resize and FourierTransform::backward /
forward (serial FFT_NOLIB build) and LDAFunctional::setxc, compiled from the
reference sources into oracle/_ref by oracle/build_ref.sh, on seeded inputs
and stores the results.
The reference's tests pin nothing on this path, so these files are the pins
for the oracle restatement (oracle/qbo.c) and for the product's basis
builder.  Usage:

    sh oracle/build_ref.sh && python tests/golden/make_golden.py [name ...]

(names: the CASES below and "lda"; all when none is given)
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


def main(names=None):
    if O.ref() is None:
        raise SystemExit("oracle/_ref/libqbref.so is not built (run oracle/build_ref.sh)")
    if not names or "lda" in names:
        make_lda()
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
