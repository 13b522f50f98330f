"""ctypes bindings for the CPU oracle (test infrastructure only).

`libqbo.so` (oracle/qbo.c) is the plain-C FP64 restatement of the
reference's algorithms; `_ref/libqbref.so` is the reference's own serial
Basis/FourierTransform code compiled from its sources by build_ref.sh (only
where those sources exist).  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg import this module, and only as the checker or
the timed CPU baseline -- the product library never calls into it.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double


def _ptr(a):
    return a.ctypes.data_as(_P) if a is not None else None


def build():
    """Compile libqbo.so (and oracle/_ref when the reference tree is present)."""
    import subprocess
    subprocess.check_call(["make", "-s", "-C", HERE, "libqbo.so"])
    subprocess.check_call([os.path.join(HERE, "build_ref.sh")])


def _load(name):
    path = os.path.join(HERE, name)
    if not os.path.exists(path):
        raise OSError(f"oracle library {path} not built")
    return ctypes.CDLL(path)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        _lib = _load("libqbo.so")
        L = _lib
        L.qbo_basis_dims.argtypes = [_P, _D, _P]
        L.qbo_basis_fill.argtypes = [_P, _D, _P, _P, _P, _P, _P, _P, _P]
        L.qbo_cell_volume.argtypes = [_P]
        L.qbo_cell_volume.restype = _D
        L.qbo_ft_create.argtypes = [_I, _I, _P, _P, _P, _P, _I, _I, _I, _I]
        L.qbo_ft_create.restype = _P
        L.qbo_ft_destroy.argtypes = [_P]
        L.qbo_ft_backward.argtypes = [_P, _P, _P]
        L.qbo_ft_forward.argtypes = [_P, _P, _P]
        L.qbo_ham_create.argtypes = [_P, _I, _P, _D, _P, _I, _P, _P, _P, _P, _P]
        L.qbo_ham_create.restype = _P
        L.qbo_ham_destroy.argtypes = [_P]
        L.qbo_ham_set_A.argtypes = [_P, _P]
        L.qbo_ham_nproj.argtypes = [_P]
        L.qbo_ham_projector.argtypes = [_P, _I, _P, _P, _P, _P]
        L.qbo_ham_set_species_tables.argtypes = [_P, _I, _I, _P, _P, _P]
        L.qbo_hpsi.argtypes = [_P, _P, _I, _I, _P, _P, _I]
        L.qbo_hpsi.restype = _D
        L.qbo_nl_apply.argtypes = [_P, _P, _I, _I, _P, _P, _I]
        L.qbo_nl_apply.restype = _D
        L.qbo_kinetic_add.argtypes = [_P, _P, _I, _I, _P]
        L.qbo_rs_mul_add.argtypes = [_P, _P, _I, _I, _P, _I]
        L.qbo_update_density.argtypes = [_P, _P, _I, _I, _P, _D, _P, _I]
        L.qbo_update_density.restype = _D
        L.qbo_current_rs.argtypes = [_P, _P, _I, _P, _I, _I, _P, _D, _P, _D, _P, _I]
        L.qbo_current_g.argtypes = [_P, _I, _P, _I, _I, _P, _P, _D, _P]
        L.qbo_etrs_step.argtypes = [_P, _P, _I, _I, _P, _D, _P, _P, _P, _I]
        L.qbo_etrs_step.restype = _D
        L.qbo_lda.argtypes = [_D, _P, _P]
        L.qbo_density_g.argtypes = [_P, _P, _D, _P]
        L.qbo_update_vhxc.argtypes = [_P, _P, _I, _P, _P, _P, _D, _P, _P]
        L.qbo_update_vhxc.restype = _D
        L.qbo_etrs_step_hxc.argtypes = [_P, _P, _I, _I, _P, _D, _P, _P, _P, _P, _I, _P, _P,
                                        _P, _I]
        L.qbo_etrs_step_hxc.restype = _D
        L.qbo_ham_get_vr.argtypes = [_P, _P]
        L.qbo_aetrs_step.argtypes = [_P, _P, _I, _I, _P, _D, _P, _P, _P, _P, _I, _P, _P, _P,
                                     _P, _I]
        L.qbo_aetrs_step.restype = _D
    return _lib


def ref():
    """The reference's own Basis/FourierTransform (None when not built)."""
    global _ref
    if _ref is None:
        try:
            _ref = _load(os.path.join("_ref", "libqbref.so"))
        except OSError:
            return None
        R = _ref
        R.qbref_basis_create.argtypes = [_P, _D, _I]
        R.qbref_basis_create.restype = _P
        R.qbref_basis_destroy.argtypes = [_P]
        R.qbref_basis_info.argtypes = [_P, _P]
        R.qbref_basis_rods.argtypes = [_P, _P, _P, _P, _P]
        R.qbref_basis_tables.argtypes = [_P, _P, _P, _P]
        R.qbref_ft_create.argtypes = [_P, _I, _I, _I]
        R.qbref_ft_create.restype = _P
        R.qbref_ft_destroy.argtypes = [_P]
        R.qbref_ft_backward.argtypes = [_P, _P, _P]
        R.qbref_ft_forward.argtypes = [_P, _P, _P]
        R.qbref_lda.argtypes = [_I, _P, _P, _P]
        R.qbref_species_load.argtypes = [ctypes.c_char_p, _D]
        R.qbref_species_load.restype = _P
        R.qbref_species_destroy.argtypes = [_P]
        R.qbref_species_info.argtypes = [_P, _P]
        R.qbref_species_wsg.argtypes = [_P, _I, _I]
        R.qbref_species_wsg.restype = _D
        R.qbref_species_vnlg.argtypes = [_P, _I, _I, _I, _P, _P]
    return _ref


def gram(c):
    """SlaterDet::gram (SlaterDet.cc:1103-1135, complex branch): columns of c
    [ngw x nst] orthonormalised as C L^{-H} with C^H C = L L^H (herk, potrf
    lower, trsm right/lower/conjugate-transpose), in FP64."""
    c = np.asarray(c, np.complex128)
    s = c.conj().T @ c
    L = np.linalg.cholesky(s)
    # X L^H = C  ->  X = C L^{-H}
    return np.linalg.solve(L.conj(), c.T).T


def ref_species_load(path, rcps=1.0):
    """A pseudopotential read and initialised by the reference's own Species
    code (handle; ref_species_destroy frees it)."""
    h = ref().qbref_species_load(path.encode(), float(rcps))
    if not h:
        raise OSError(f"reference Species could not read {path}")
    return h


def ref_species_destroy(h):
    ref().qbref_species_destroy(h)


def ref_species_info(h):
    """[lmax, llocal, nchannels, nlm, zval, nquad, ultrasoft, 0]"""
    info = np.zeros(8, np.int32)
    ref().qbref_species_info(h, _ptr(info))
    return info


def ref_species_wsg(h, l, ic):
    return float(ref().qbref_species_wsg(h, int(l), int(ic)))


def ref_species_vnlg(h, l, ic, g):
    """Species::dvnlg(l, ic, g) values for the |G| values g."""
    g = np.ascontiguousarray(g, np.float64)
    v = np.zeros_like(g)
    ref().qbref_species_vnlg(h, int(l), int(ic), g.size, _ptr(g), _ptr(v))
    return v


def ref_lda(rho):
    """The reference's LDAFunctional::setxc: (exc, vxc) for rho."""
    rho = np.ascontiguousarray(rho, np.float64)
    exc = np.zeros_like(rho)
    vxc = np.zeros_like(rho)
    ref().qbref_lda(rho.size, _ptr(rho), _ptr(exc), _ptr(vxc))
    return exc, vxc


class Basis:
    """Full-sphere plane-wave basis (restated Basis::resize)."""

    def __init__(self, a, ecut, use_ref=False):
        self.a = np.ascontiguousarray(a, dtype=np.float64).reshape(9)
        self.ecut = float(ecut)
        info = np.zeros(12, dtype=np.int32)
        if use_ref:
            R = ref()
            h = R.qbref_basis_create(_ptr(self.a), self.ecut, 1)
            R.qbref_basis_info(h, _ptr(info))
        else:
            lib().qbo_basis_dims(_ptr(self.a), self.ecut, _ptr(info))
        self.ngw = int(info[0])
        self.nrods = int(info[1])
        self.np = tuple(int(x) for x in info[2:5])
        self.idxmin = tuple(int(x) for x in info[5:8])
        self.idxmax = tuple(int(x) for x in info[8:11])
        self.rod_h = np.zeros(self.nrods, np.int32)
        self.rod_k = np.zeros(self.nrods, np.int32)
        self.rod_lmin = np.zeros(self.nrods, np.int32)
        self.rod_size = np.zeros(self.nrods, np.int32)
        self.idx = np.zeros(3 * self.ngw, np.int32)
        self.kpg2 = np.zeros(self.ngw)
        self.kpgx = np.zeros(3 * self.ngw)
        if use_ref:
            R.qbref_basis_rods(h, _ptr(self.rod_h), _ptr(self.rod_k),
                               _ptr(self.rod_lmin), _ptr(self.rod_size))
            R.qbref_basis_tables(h, _ptr(self.idx), _ptr(self.kpg2), _ptr(self.kpgx))
            R.qbref_basis_destroy(h)
        else:
            lib().qbo_basis_fill(_ptr(self.a), self.ecut, _ptr(self.rod_h), _ptr(self.rod_k),
                                 _ptr(self.rod_lmin), _ptr(self.rod_size), _ptr(self.idx),
                                 _ptr(self.kpg2), _ptr(self.kpgx))
        self.omega = float(lib().qbo_cell_volume(_ptr(self.a)))

    @property
    def ntrans0(self):
        return max(abs(self.idxmax[1]), abs(self.idxmin[1])) + 1


class FT:
    """Restated FourierTransform (complex basis, one process)."""

    def __init__(self, basis, np0, np1, np2):
        self.basis = basis
        self.shape = (np0, np1, np2)
        self.n012 = np0 * np1 * np2
        self.h = lib().qbo_ft_create(basis.ngw, basis.nrods, _ptr(basis.rod_h),
                                     _ptr(basis.rod_k), _ptr(basis.rod_lmin),
                                     _ptr(basis.rod_size), np0, np1, np2, basis.ntrans0)

    def __del__(self):
        if getattr(self, "h", None):
            lib().qbo_ft_destroy(self.h)
            self.h = None

    def backward(self, c):
        c = np.ascontiguousarray(c, dtype=np.complex128)
        f = np.zeros(self.n012, np.complex128)
        lib().qbo_ft_backward(self.h, _ptr(c), _ptr(f))
        return f

    def forward(self, f):
        f = np.array(f, dtype=np.complex128, copy=True)
        c = np.zeros(self.basis.ngw, np.complex128)
        lib().qbo_ft_forward(self.h, _ptr(f), _ptr(c))
        return c


class RefFT:
    """The reference's own FourierTransform (oracle/_ref), for pinning."""

    def __init__(self, a, ecut, np0, np1, np2):
        R = ref()
        self.a = np.ascontiguousarray(a, dtype=np.float64).reshape(9)
        self.hb = R.qbref_basis_create(_ptr(self.a), float(ecut), 1)
        info = np.zeros(12, np.int32)
        R.qbref_basis_info(self.hb, _ptr(info))
        self.ngw = int(info[0])
        self.n012 = np0 * np1 * np2
        self.h = R.qbref_ft_create(self.hb, np0, np1, np2)

    def __del__(self):
        R = ref()
        if getattr(self, "h", None):
            R.qbref_ft_destroy(self.h)
            R.qbref_basis_destroy(self.hb)
            self.h = None

    def backward(self, c):
        c = np.ascontiguousarray(c, dtype=np.complex128)
        f = np.zeros(self.n012, np.complex128)
        ref().qbref_ft_backward(self.h, _ptr(c), _ptr(f))
        return f

    def forward(self, f):
        f = np.array(f, dtype=np.complex128, copy=True)
        c = np.zeros(self.ngw, np.complex128)
        ref().qbref_ft_forward(self.h, _ptr(f), _ptr(c))
        return c


class Ham:
    """Restated Hamiltonian (kinetic + local + KB nonlocal) and ETRS step."""

    def __init__(self, ft, v_r, species):
        """species: list of dicts {tau: (na,3), lmax, rc, wt: [w0,w1,w2]} (the
        synthetic radial form) or {tau, twnl: (npr, ngw), lproj: (npr,), wt:
        (npr,)} (projector tables as NonLocalPotential::update_twnl builds
        them, evaluated at |k+G-A| for the A in force)."""
        self.ft = ft
        b = ft.basis
        self.v_r = np.ascontiguousarray(v_r, dtype=np.float64)
        nsp = len(species)
        tables = [("twnl" in s) for s in species]
        self.na = np.array([len(s["tau"]) for s in species], np.int32)
        self.lmax = np.array([-1 if t else s["lmax"] for s, t in zip(species, tables)], np.int32)
        self.rc = np.array([s.get("rc", 1.0) for s in species], np.float64)
        self.wt = np.zeros(3 * max(nsp, 1))
        for i, s in enumerate(species):
            if tables[i]:
                continue
            w = list(s["wt"]) + [0.0] * 3
            self.wt[3 * i:3 * i + 3] = w[:3]
        self.tau = np.ascontiguousarray(
            np.concatenate([np.asarray(s["tau"], np.float64).reshape(-1) for s in species])
            if nsp else np.zeros(3), dtype=np.float64)
        self.h = lib().qbo_ham_create(ft.h, b.ngw, _ptr(b.kpgx), b.omega, _ptr(self.v_r),
                                      nsp, _ptr(self.na), _ptr(self.lmax), _ptr(self.rc),
                                      _ptr(self.wt), _ptr(self.tau))
        for i, s in enumerate(species):
            if tables[i]:
                tw = np.ascontiguousarray(s["twnl"], np.float64)
                lp = np.ascontiguousarray(s["lproj"], np.int32)
                w = np.ascontiguousarray(s["wt"], np.float64)
                lib().qbo_ham_set_species_tables(self.h, i, len(lp), _ptr(lp), _ptr(w), _ptr(tw))

    def __del__(self):
        if getattr(self, "h", None):
            lib().qbo_ham_destroy(self.h)
            self.h = None

    def set_A(self, A):
        A = np.ascontiguousarray(A, dtype=np.float64)
        lib().qbo_ham_set_A(self.h, _ptr(A))

    def nproj(self):
        return lib().qbo_ham_nproj(self.h)

    def projector(self, p):
        t = np.zeros(self.ft.basis.ngw)
        l = ctypes.c_int()
        w = ctypes.c_double()
        tau = np.zeros(3)
        lib().qbo_ham_projector(self.h, p, _ptr(t), ctypes.byref(l), ctypes.byref(w), _ptr(tau))
        return t, l.value, w.value, tau

    def hpsi(self, c, occ, nthreads=1):
        c = np.asfortranarray(c, dtype=np.complex128)
        ngw, nst = c.shape
        occ = np.ascontiguousarray(occ, dtype=np.float64)
        cp = np.zeros_like(c, order="F")
        enl = lib().qbo_hpsi(self.h, _ptr(c), ngw, nst, _ptr(occ), _ptr(cp), nthreads)
        return cp, enl

    def parts(self, c, occ, nthreads=1):
        """(nonlocal, kinetic, local) contributions separately."""
        c = np.asfortranarray(c, dtype=np.complex128)
        ngw, nst = c.shape
        occ = np.ascontiguousarray(occ, dtype=np.float64)
        out = []
        cp = np.zeros_like(c, order="F")
        enl = lib().qbo_nl_apply(self.h, _ptr(c), ngw, nst, _ptr(occ), _ptr(cp), nthreads)
        out.append(cp)
        cp = np.zeros_like(c, order="F")
        lib().qbo_kinetic_add(self.h, _ptr(c), ngw, nst, _ptr(cp))
        out.append(cp)
        cp = np.zeros_like(c, order="F")
        lib().qbo_rs_mul_add(self.h, _ptr(c), ngw, nst, _ptr(cp), nthreads)
        out.append(cp)
        return out, enl

    def etrs_step(self, psi, occ, dt, A_t, A_tdt, want_rho=False, nthreads=1):
        psi = np.asfortranarray(psi, dtype=np.complex128).copy(order="F")
        ngw, nst = psi.shape
        occ = np.ascontiguousarray(occ, dtype=np.float64)
        rho = np.zeros(self.ft.n012) if want_rho else None
        A_t = np.ascontiguousarray(A_t, dtype=np.float64)
        A_tdt = np.ascontiguousarray(A_tdt, dtype=np.float64)
        nel = lib().qbo_etrs_step(self.h, _ptr(psi), ngw, nst, _ptr(occ), float(dt),
                                  _ptr(A_t), _ptr(A_tdt), _ptr(rho), nthreads)
        return psi, rho, nel

    def aetrs_step(self, psi, occ, dt, A_t, A_tdt, hxc=None, nthreads=1):
        """AETRS step (approximated_ stepper); the stored potentials live on
        this object (reset_aetrs clears them).  hxc: an Hxc object for the
        self-consistent loop top, or None for a fixed potential."""
        n012 = self.ft.n012
        if getattr(self, "_vhist", None) is None:
            self.reset_aetrs()
        psi = np.asfortranarray(psi, dtype=np.complex128).copy(order="F")
        ngw, nst = psi.shape
        occ = np.ascontiguousarray(occ, dtype=np.float64)
        A_t = np.ascontiguousarray(A_t, dtype=np.float64)
        A_tdt = np.ascontiguousarray(A_tdt, dtype=np.float64)
        st = ctypes.c_int(self._stored)
        if hxc is None:
            args = (None, None, 0, None, None)
        else:
            args = (hxc.vft.h, _ptr(hxc.vbasis.kpg2), hxc.vbasis.ngw, _ptr(hxc.vion),
                    _ptr(hxc.rhopst))
        lib().qbo_aetrs_step(self.h, _ptr(psi), ngw, nst, _ptr(occ), float(dt), _ptr(A_t),
                             _ptr(A_tdt), *args, _ptr(self._vhist), ctypes.byref(st), nthreads)
        self._stored = st.value
        assert n012 == self._vhist.size // 3
        return psi

    def reset_aetrs(self):
        self._vhist = np.zeros(3 * self.ft.n012)
        self._stored = 0

    def etrs_step_hxc(self, psi, occ, dt, A_t, A_tdt, hxc, want_rho=False, nthreads=1):
        """ETRS step with v_r rebuilt by update_vhxc (hxc: an Hxc object)."""
        psi = np.asfortranarray(psi, dtype=np.complex128).copy(order="F")
        ngw, nst = psi.shape
        occ = np.ascontiguousarray(occ, dtype=np.float64)
        rho = np.zeros(self.ft.n012) if want_rho else None
        A_t = np.ascontiguousarray(A_t, dtype=np.float64)
        A_tdt = np.ascontiguousarray(A_tdt, dtype=np.float64)
        nel = lib().qbo_etrs_step_hxc(self.h, _ptr(psi), ngw, nst, _ptr(occ), float(dt),
                                      _ptr(A_t), _ptr(A_tdt), hxc.vft.h, _ptr(hxc.vbasis.kpg2),
                                      hxc.vbasis.ngw, _ptr(hxc.vion), _ptr(hxc.rhopst),
                                      _ptr(rho), nthreads)
        return psi, rho, nel

    def v_r_now(self):
        v = np.zeros(self.ft.n012)
        lib().qbo_ham_get_vr(self.h, _ptr(v))
        return v


def lda(rho):
    """(e_xc, v_xc) per grid point, Perdew-Zunger LDA (scalar loop)."""
    e = ctypes.c_double()
    v = ctypes.c_double()
    rho = np.asarray(rho, np.float64).reshape(-1)
    E = np.zeros_like(rho)
    V = np.zeros_like(rho)
    for i, r in enumerate(rho):
        lib().qbo_lda(float(r), ctypes.byref(e), ctypes.byref(v))
        E[i] = e.value
        V[i] = v.value
    return E, V


class Hxc:
    """Density-basis transform and ionic terms for update_vhxc."""

    def __init__(self, vbasis, np0, np1, np2, vion_g, rhopst_g=None):
        self.vbasis = vbasis
        self.vft = FT(vbasis, np0, np1, np2)
        self.vion = np.ascontiguousarray(np.asarray(vion_g, np.complex128))
        self.rhopst = (np.ascontiguousarray(np.asarray(rhopst_g, np.complex128))
                       if rhopst_g is not None else None)

    def density_g(self, rho):
        rho = np.ascontiguousarray(rho, np.float64)
        rg = np.zeros(self.vbasis.ngw, np.complex128)
        lib().qbo_density_g(self.vft.h, _ptr(rho), self.vbasis.omega, _ptr(rg))
        return rg

    def update_vhxc(self, rho):
        """(v_r, {ehart, exc, eps})"""
        rho = np.ascontiguousarray(rho, np.float64)
        v = np.zeros(self.vft.n012)
        en = np.zeros(3)
        lib().qbo_update_vhxc(self.vft.h, _ptr(self.vbasis.kpg2), self.vbasis.ngw,
                              _ptr(self.vion), _ptr(self.rhopst), _ptr(rho), self.vbasis.omega,
                              _ptr(v), _ptr(en))
        return v, dict(zip(("ehart", "exc", "eps"), en.tolist()))


def update_density(ft, c, occ, nthreads=1):
    c = np.asfortranarray(c, dtype=np.complex128)
    ngw, nst = c.shape
    occ = np.ascontiguousarray(occ, dtype=np.float64)
    rho = np.zeros(ft.n012)
    nel = lib().qbo_update_density(ft.h, _ptr(c), ngw, nst, _ptr(occ), ft.basis.omega,
                                   _ptr(rho), nthreads)
    return rho, nel


def current_rs(ft, c, occ, A, nel):
    c = np.asfortranarray(c, dtype=np.complex128)
    ngw, nst = c.shape
    occ = np.ascontiguousarray(occ, dtype=np.float64)
    A = np.ascontiguousarray(A, dtype=np.float64)
    J = np.zeros(3)
    lib().qbo_current_rs(ft.h, _ptr(ft.basis.kpgx), ngw, _ptr(c), ngw, nst, _ptr(occ),
                         ft.basis.omega, _ptr(A), float(nel), _ptr(J), 1)
    return J


def current_g(basis, c, occ, A, nel):
    c = np.asfortranarray(c, dtype=np.complex128)
    ngw, nst = c.shape
    occ = np.ascontiguousarray(occ, dtype=np.float64)
    A = np.ascontiguousarray(A, dtype=np.float64)
    J = np.zeros(3)
    lib().qbo_current_g(_ptr(basis.kpgx), ngw, _ptr(c), ngw, nst, _ptr(occ), _ptr(A),
                        float(nel), _ptr(J))
    return J
