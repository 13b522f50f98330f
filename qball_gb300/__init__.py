"""qball-gb300: GB300-native Kohn-Sham H|psi> and ETRS propagation.

The compute path is libqbg.so (hand-written sm_103a CUDA behind the C ABI of
include/qbg.h).  This module is the thin host mirror of the reference's
operator surface over that ABI:

  Basis                         Basis::resize              (Basis.cc:302)
  FourierTransform              FourierTransform           (FourierTransform.h:136)
    .backward / .forward                                   (FourierTransform.cc:529,542)
  Hamiltonian.hpsi              EnergyFunctional::energy(compute_hpsi=true)
                                                           (EnergyFunctional.cc:1128)
  Hamiltonian.update_density    ChargeDensity::update_density (ChargeDensity.cc:276)
  Hamiltonian.current           CurrentDensity::update_current (CurrentDensity.cc:39)
  Hamiltonian.etrs_step         ExponentialWavefunctionStepper::preupdate+update
                                                           (ExponentialWavefunctionStepper.cc:153,241)

Device arrays are torch tensors (torch is used only for device memory and
streams) or raw integer device pointers.  A wavefunction block is a complex
tensor of shape [nst, ld] -- column-major [ld x nst] in the reference's
terms.  There is no CPU fallback: if libqbg.so is missing or no GPU is
present, the operators raise.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libqbg.so")

QBG_PREC_FP64 = 0
QBG_PREC_MIXED = 1
QBG_PREC_MIXED_FFT64 = 2
QBG_PREC_MIXED_NL64 = 3
QBG_PREC_MIXED_DF32 = 4
QBG_GEMM_SIMT = 0
QBG_GEMM_OZAKI = 1
PRECISIONS = {"fp64": QBG_PREC_FP64, "mixed": QBG_PREC_MIXED,
              "mixed_fft64": QBG_PREC_MIXED_FFT64, "mixed_nl64": QBG_PREC_MIXED_NL64,
              "mixed_df32": QBG_PREC_MIXED_DF32}
_STATUS = {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "unsupported",
           4: "CUDA error", 5: "timeout", 6: "diverged", 7: "bad state"}

_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double

# entry points declared in include/qbg.h: name -> argtypes
ABI = {
    "qbg_last_error": [],
    "qbg_version": [],
    "qbg_basis_dims": [_P, _D, _P],
    "qbg_basis_fill": [_P, _D, _P, _P, _P, _P, _P, _P, _P],
    "qbg_plan_create": [_P, _I, _I, _I, _I, _P],
    "qbg_plan_destroy": [_P],
    "qbg_plan_set_chunk": [_P, _I],
    "qbg_plan_set_fp64_gemm": [_P, _I, _I],
    "qbg_backward": [_P, _P, _I, _P, _I, _P],
    "qbg_backward_noalloc": [_P, _P, _I, _P, _I, _P],
    "qbg_forward": [_P, _P, _P, _I, _I, _P],
    "qbg_set_vlocal": [_P, _P],
    "qbg_get_vlocal": [_P, _P],
    "qbg_set_nonlocal": [_P, _I, _P, _P, _P, _P, _P],
    "qbg_set_nonlocal_tables": [_P, _I, _P, _P, _P, _P, _P, _P],
    "qbg_set_vector_potential": [_P, _P],
    "qbg_hpsi": [_P, _P, _I, _P, _I, _P, _P, _P],
    "qbg_density": [_P, _P, _I, _I, _P, _D, _P, _P, _P],
    "qbg_current": [_P, _P, _I, _I, _P, _D, _P, _P],
    "qbg_set_density_basis": [_P, _P],
    "qbg_set_ionic_terms": [_P, _P, _P],
    "qbg_density_g": [_P, _P, _P, _P],
    "qbg_update_vhxc": [_P, _P, _P, _P],
    "qbg_set_selfconsistent": [_P, _I],
    "qbg_etrs_step": [_P, _P, _I, _I, _P, _D, _P, _P, _P, _P, _P],
    "qbg_gram": [_P, _P, _I, _I, _P],
    "qbg_set_aetrs": [_P, _I],
    "qbg_etrs_adjoint_step": [_P, _P, _I, _I, _P, _D, _P, _P, _P, _P, _P, _P, _P],
    "qbg_td_create": [_P, _I, _I, _P, _D, _I, _I, _P],
    "qbg_td_forward": [_P, _P, _P, _P, _P],
    "qbg_td_backward": [_P, _P, _P, _P, _P, _P, _P],
    "qbg_td_destroy": [_P],
    "qbg_etrs_graph_create": [_I, _P, _P, _P, _P, _P, _D, _P, _P],
    "qbg_etrs_graph_launch": [_P, _P],
    "qbg_etrs_graph_check": [_P],
    "qbg_etrs_graph_destroy": [_P],
    "qbg_plan_autotune": [_P, _P, _I, _I, _P, _P, _P],
    "qbg_plan_set_transform_config": [_P, _I, _I, _I, _I],
    "qbg_plan_get_transform_config": [_P, _P],
    "qbg_selftest_wait_timeout": [_I],
    "qbg_plan_set_wait_polls": [_P, _I],
    "qbg_launch_count": [_P, _P],
    "qbg_profile": [_P, _I],
    "qbg_profile_read": [_P, _P, _P, _I],
    "qbg_phase_name": [_I],
}
NPHASE = 14


class QbgError(RuntimeError):
    pass


class _BasisDesc(ctypes.Structure):
    _fields_ = [("ngw", _I), ("nrods", _I), ("rod_h", _P), ("rod_k", _P),
                ("rod_lmin", _P), ("rod_size", _P), ("kpgx", _P), ("omega", _D)]


_lib = None


def lib():
    """Load libqbg.so (build it first with qball_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise QbgError(f"{LIBPATH} is not built; run python -m qball_gb300.build")
        L = ctypes.CDLL(LIBPATH)
        for name, args in ABI.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = (ctypes.c_char_p if name in ("qbg_last_error", "qbg_version", "qbg_phase_name")
                          else _I)
        _lib = L
    return _lib


def _check(status, what):
    if status != 0:
        msg = lib().qbg_last_error().decode(errors="replace")
        raise QbgError(f"{what}: {_STATUS.get(status, status)}: {msg}")


def _np_ptr(a):
    return a.ctypes.data_as(_P) if a is not None else None


def _dev_ptr(x):
    if x is None:
        return None
    if isinstance(x, int):
        return _P(x)
    if hasattr(x, "is_contiguous") and not x.is_contiguous():
        raise QbgError("device arrays must be contiguous (row-major [nst][ld] for states)")
    return _P(x.data_ptr())


def _stream_ptr(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return _P(stream)
    return _P(stream.cuda_stream)


def cubic_cell(L):
    return np.diag([float(L)] * 3).reshape(9)


class Basis:
    """Full-sphere plane-wave basis at k=0 (Basis::resize, Basis.cc:302-700).

    cell: 9 floats (a0, a1, a2) or a scalar edge L of a cubic cell;
    ecut in Hartree.
    """

    def __init__(self, cell, ecut):
        a = cubic_cell(cell) if np.isscalar(cell) else np.ascontiguousarray(cell, np.float64).reshape(9)
        self.a = a
        self.ecut = float(ecut)
        info = np.zeros(12, np.int32)
        _check(lib().qbg_basis_dims(_np_ptr(a), self.ecut, _np_ptr(info)), "qbg_basis_dims")
        self.ngw, self.nrods = int(info[0]), int(info[1])
        self.np = tuple(int(v) for v in info[2:5])
        self.idxmin = tuple(int(v) for v in info[5:8])
        self.idxmax = tuple(int(v) for v in info[8:11])
        self.rod_h = np.zeros(self.nrods, np.int32)
        self.rod_k = np.zeros(self.nrods, np.int32)
        self.rod_lmin = np.zeros(self.nrods, np.int32)
        self.rod_size = np.zeros(self.nrods, np.int32)
        self.idx = np.zeros(3 * self.ngw, np.int32)
        self.kpg2 = np.zeros(self.ngw)
        self.kpgx = np.zeros(3 * self.ngw)
        _check(lib().qbg_basis_fill(_np_ptr(a), self.ecut, _np_ptr(self.rod_h), _np_ptr(self.rod_k),
                                    _np_ptr(self.rod_lmin), _np_ptr(self.rod_size), _np_ptr(self.idx),
                                    _np_ptr(self.kpg2), _np_ptr(self.kpgx)), "qbg_basis_fill")
        a3 = a.reshape(3, 3)
        self.omega = float(np.dot(a3[0], np.cross(a3[1], a3[2])))


class FourierTransform:
    """A plan: FourierTransform(basis, np0, np1, np2) plus the operators that
    share its tables.  precision: "fp64" (plain) or "mixed"."""

    def __init__(self, basis, np0, np1, np2, precision="fp64"):
        self.basis = basis
        self.shape = (int(np0), int(np1), int(np2))
        self.n012 = int(np0) * int(np1) * int(np2)
        self.precision = precision
        if precision not in PRECISIONS:
            raise QbgError(f"unknown precision {precision!r}; one of {sorted(PRECISIONS)}")
        prec = PRECISIONS[precision]
        d = _BasisDesc(basis.ngw, basis.nrods, _np_ptr(basis.rod_h), _np_ptr(basis.rod_k),
                       _np_ptr(basis.rod_lmin), _np_ptr(basis.rod_size), _np_ptr(basis.kpgx),
                       basis.omega)
        h = _P()
        _check(lib().qbg_plan_create(ctypes.byref(d), int(np0), int(np1), int(np2), prec,
                                     ctypes.byref(h)), "qbg_plan_create")
        self.h = h
        self.chunk = self.transform_config()["chunk"]  # plan default: 96 on 120 x 120 planes, else 32
        self.fp64_gemm, self.oz_slices = "ozaki", 7  # plan default

    def close(self):
        if getattr(self, "h", None):
            lib().qbg_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def profile(self, enable=True):
        _check(lib().qbg_profile(self.h, 1 if enable else 0), "qbg_profile")

    def profile_read(self):
        ms = np.zeros(NPHASE)
        n = np.zeros(NPHASE, np.int64)
        _check(lib().qbg_profile_read(self.h, _np_ptr(ms), _np_ptr(n), NPHASE), "qbg_profile_read")
        return {lib().qbg_phase_name(i).decode(): (float(ms[i]), int(n[i])) for i in range(NPHASE)}

    def autotune(self, psi, occ, stream=None):
        """Pick the states-per-launch-group that makes H|psi> fastest."""
        o = np.ascontiguousarray(occ, np.float64)
        ch = ctypes.c_int()
        _check(lib().qbg_plan_autotune(self.h, _dev_ptr(psi), int(psi.shape[-1]),
                                       int(psi.shape[0]), _np_ptr(o), _stream_ptr(stream),
                                       ctypes.byref(ch)), "qbg_plan_autotune")
        self.chunk = ch.value
        return ch.value

    def set_fp64_gemm(self, mode="ozaki", slices=7):
        """Projector GEMMs of the plain FP64 form: "ozaki" (FP64-accurate on
        the tensor cores, `slices` 7-bit digit planes, the default) or
        "simt" (FP64 FMAs)."""
        m = {"simt": QBG_GEMM_SIMT, "ozaki": QBG_GEMM_OZAKI}[mode]
        _check(lib().qbg_plan_set_fp64_gemm(self.h, m, int(slices)), "qbg_plan_set_fp64_gemm")
        self.fp64_gemm, self.oz_slices = mode, int(slices)

    def set_transform_config(self, radix_order=0, prime_factor=1, fused=2, lane_group=1):
        """fused: 2 whole-plane kernel on 120 x 120 planes (band-row kernel
        elsewhere), 1 band-row fused kernel, 0 separate x, y, x kernels."""
        _check(lib().qbg_plan_set_transform_config(self.h, int(radix_order), int(prime_factor),
                                                   int(fused), int(lane_group)),
               "qbg_plan_set_transform_config")

    def transform_config(self):
        """{chunk, radix_order, prime_factor, fused, lane_group}"""
        c = np.zeros(5, np.int32)
        _check(lib().qbg_plan_get_transform_config(self.h, _np_ptr(c)),
               "qbg_plan_get_transform_config")
        return dict(zip(("chunk", "radix_order", "prime_factor", "fused", "lane_group"),
                        c.tolist()))

    def set_chunk(self, n):
        _check(lib().qbg_plan_set_chunk(self.h, int(n)), "qbg_plan_set_chunk")
        self.chunk = int(n)

    def set_wait_polls(self, polls=-1):
        """Poll limit of the tensor-core GEMMs' pipeline waits (-1: default;
        0: every such wait expires at once, for tests of the timeout path)."""
        _check(lib().qbg_plan_set_wait_polls(self.h, int(polls)), "qbg_plan_set_wait_polls")

    def launches(self):
        c = ctypes.c_longlong()
        _check(lib().qbg_launch_count(self.h, ctypes.byref(c)), "qbg_launch_count")
        return c.value

    def gram(self, psi, nst=None, ld=None, stream=None):
        """SlaterDet::gram: orthonormalise the device states psi in place."""
        n = psi.shape[0] if nst is None else nst
        ldv = psi.shape[-1] if ld is None else ld
        _check(lib().qbg_gram(self.h, _dev_ptr(psi), ldv, n, _stream_ptr(stream)), "qbg_gram")

    # ---- FourierTransform::backward / forward, batched over states
    def backward(self, c, f, nbatch=None, ldc=None, stream=None):
        nb = c.shape[0] if nbatch is None else nbatch
        ld = c.shape[-1] if ldc is None else ldc
        _check(lib().qbg_backward(self.h, _dev_ptr(c), ld, _dev_ptr(f), nb, _stream_ptr(stream)),
               "qbg_backward")

    def forward(self, f, c, nbatch=None, ldc=None, stream=None):
        nb = c.shape[0] if nbatch is None else nbatch
        ld = c.shape[-1] if ldc is None else ldc
        _check(lib().qbg_forward(self.h, _dev_ptr(f), _dev_ptr(c), ld, nb, _stream_ptr(stream)),
               "qbg_forward")


class Hamiltonian(FourierTransform):
    """EnergyFunctional-shaped operator set on one plan."""

    def set_vlocal(self, v_r):
        v = np.ascontiguousarray(v_r, np.float64) if isinstance(v_r, np.ndarray) else v_r
        ptr = _np_ptr(v) if isinstance(v, np.ndarray) else _dev_ptr(v)
        _check(lib().qbg_set_vlocal(self.h, ptr), "qbg_set_vlocal")

    def get_vlocal(self, out=None):
        """The FP64 v_r in use (numpy array, or into the device tensor out)."""
        v = np.zeros(self.n012) if out is None else out
        ptr = _np_ptr(v) if isinstance(v, np.ndarray) else _dev_ptr(v)
        _check(lib().qbg_get_vlocal(self.h, ptr), "qbg_get_vlocal")
        return v

    def set_nonlocal(self, species):
        """species: list of {tau: (na,3), lmax, rc, wt: [w_s, w_p, w_d]} (the
        synthetic radial form), or of {tau, twnl: (npr, ngw), lproj: (npr,),
        wt: (npr,)} (projector tables of real pseudopotentials as
        NonLocalPotential::update_twnl builds them, for the A in force)."""
        if species and all("twnl" in s for s in species):
            return self.set_nonlocal_tables(species)
        nsp = len(species)
        na = np.array([len(s["tau"]) for s in species], np.int32)
        lmax = np.array([s["lmax"] for s in species], np.int32)
        rc = np.array([s["rc"] for s in species], np.float64)
        wt = np.zeros(3 * max(nsp, 1))
        for i, s in enumerate(species):
            w = list(s["wt"]) + [0.0] * 3
            wt[3 * i:3 * i + 3] = w[:3]
        tau = (np.ascontiguousarray(np.concatenate([np.asarray(s["tau"], np.float64).reshape(-1)
                                                    for s in species]))
               if nsp else np.zeros(3))
        _check(lib().qbg_set_nonlocal(self.h, nsp, _np_ptr(na), _np_ptr(lmax), _np_ptr(rc),
                                      _np_ptr(wt), _np_ptr(tau)), "qbg_set_nonlocal")

    def set_nonlocal_tables(self, species):
        """Projector tables (qbg_set_nonlocal_tables): per species tau (na,3),
        twnl (npr, ngw) at |k+G-A|, lproj (npr,), wt (npr,) in Hartree."""
        nsp = len(species)
        na = np.array([len(s["tau"]) for s in species], np.int32)
        npr = np.array([len(s["lproj"]) for s in species], np.int32)
        lproj = np.ascontiguousarray(np.concatenate([np.asarray(s["lproj"], np.int32)
                                                     for s in species]), np.int32)
        wt = np.ascontiguousarray(np.concatenate([np.asarray(s["wt"], np.float64)
                                                  for s in species]), np.float64)
        twnl = np.ascontiguousarray(np.concatenate([np.asarray(s["twnl"], np.float64)
                                                    .reshape(-1, self.basis.ngw)
                                                    for s in species]), np.float64)
        tau = np.ascontiguousarray(np.concatenate([np.asarray(s["tau"], np.float64).reshape(-1)
                                                   for s in species]), np.float64)
        _check(lib().qbg_set_nonlocal_tables(self.h, nsp, _np_ptr(na), _np_ptr(npr),
                                             _np_ptr(lproj), _np_ptr(wt), _np_ptr(twnl),
                                             _np_ptr(tau)), "qbg_set_nonlocal_tables")

    # ---- Hartree + xc (EnergyFunctional::update_vhxc)
    def set_density_basis(self, vbasis):
        """vbasis: Basis of the density sphere (ecutden, 4 ecut by default) that
        fits this plan's grid."""
        d = _BasisDesc(vbasis.ngw, vbasis.nrods, _np_ptr(vbasis.rod_h), _np_ptr(vbasis.rod_k),
                       _np_ptr(vbasis.rod_lmin), _np_ptr(vbasis.rod_size), _np_ptr(vbasis.kpgx),
                       vbasis.omega)
        _check(lib().qbg_set_density_basis(self.h, ctypes.byref(d)), "qbg_set_density_basis")
        self.vbasis = vbasis

    def set_ionic_terms(self, vion_g, rhopst_g=None):
        """vion_g, rhopst_g: complex numpy arrays [ngv] on the density basis."""
        v = np.ascontiguousarray(np.asarray(vion_g, np.complex128).view(np.float64))
        r = (np.ascontiguousarray(np.asarray(rhopst_g, np.complex128).view(np.float64))
             if rhopst_g is not None else None)
        _check(lib().qbg_set_ionic_terms(self.h, _np_ptr(v), _np_ptr(r)), "qbg_set_ionic_terms")

    def density_g(self, rho, rhog, stream=None):
        _check(lib().qbg_density_g(self.h, _dev_ptr(rho), _dev_ptr(rhog), _stream_ptr(stream)),
               "qbg_density_g")

    def update_vhxc(self, rho, want_energies=False, stream=None):
        """Returns {ehart, exc, eps} when want_energies."""
        en = np.zeros(3)
        _check(lib().qbg_update_vhxc(self.h, _dev_ptr(rho), _np_ptr(en) if want_energies else None,
                                     _stream_ptr(stream)), "qbg_update_vhxc")
        return dict(zip(("ehart", "exc", "eps"), en.tolist())) if want_energies else None

    def set_aetrs(self, on=True):
        """Approximated ETRS (the reference stepper's AETRS option)."""
        _check(lib().qbg_set_aetrs(self.h, 1 if on else 0), "qbg_set_aetrs")

    def set_selfconsistent(self, on=True):
        _check(lib().qbg_set_selfconsistent(self.h, 1 if on else 0), "qbg_set_selfconsistent")

    def set_vector_potential(self, A):
        A = np.ascontiguousarray(A, np.float64)
        _check(lib().qbg_set_vector_potential(self.h, _np_ptr(A)), "qbg_set_vector_potential")

    def hpsi(self, psi, out, occ=None, want_enl=False, nst=None, ld=None, stream=None):
        n = psi.shape[0] if nst is None else nst
        ldv = psi.shape[-1] if ld is None else ld
        o = np.ascontiguousarray(occ, np.float64) if occ is not None else None
        e = ctypes.c_double()
        _check(lib().qbg_hpsi(self.h, _dev_ptr(psi), ldv, _dev_ptr(out), n, _np_ptr(o),
                              ctypes.byref(e) if want_enl else None, _stream_ptr(stream)),
               "qbg_hpsi")
        return e.value if want_enl else None

    def update_density(self, psi, occ, rho, weight=1.0, nst=None, ld=None, stream=None):
        n = psi.shape[0] if nst is None else nst
        ldv = psi.shape[-1] if ld is None else ld
        o = np.ascontiguousarray(occ, np.float64)
        nel = ctypes.c_double()
        _check(lib().qbg_density(self.h, _dev_ptr(psi), ldv, n, _np_ptr(o), float(weight),
                                 _dev_ptr(rho), ctypes.byref(nel), _stream_ptr(stream)),
               "qbg_density")
        return nel.value

    def current(self, psi, occ, nel, nst=None, ld=None, stream=None):
        n = psi.shape[0] if nst is None else nst
        ldv = psi.shape[-1] if ld is None else ld
        o = np.ascontiguousarray(occ, np.float64)
        J = np.zeros(3)
        _check(lib().qbg_current(self.h, _dev_ptr(psi), ldv, n, _np_ptr(o), float(nel),
                                 _np_ptr(J), _stream_ptr(stream)), "qbg_current")
        return J

    def etrs_step(self, psi, occ, dt, A_t=None, A_tdt=None, rho=None, want_nel=False,
                  nst=None, ld=None, stream=None):
        n = psi.shape[0] if nst is None else nst
        ldv = psi.shape[-1] if ld is None else ld
        o = np.ascontiguousarray(occ, np.float64)
        at = np.ascontiguousarray(A_t, np.float64) if A_t is not None else None
        atd = np.ascontiguousarray(A_tdt, np.float64) if A_tdt is not None else None
        nel = ctypes.c_double()
        _check(lib().qbg_etrs_step(self.h, _dev_ptr(psi), ldv, n, _np_ptr(o), float(dt),
                                   _np_ptr(at), _np_ptr(atd), _dev_ptr(rho),
                                   ctypes.byref(nel) if want_nel else None, _stream_ptr(stream)),
               "qbg_etrs_step")
        return nel.value if want_nel else None

    def etrs_adjoint_step(self, psi_n, lam, dt, A_n=None, A_np1=None, e=None, grad_v=None,
                          want_grad_a=False, stream=None):
        """lam <- (adjoint of one fixed-potential ETRS step) lam; grad_v
        (device, N doubles) accumulates dL/dv(r); returns [dL/da_n,
        dL/da_{n+1}] along e when want_grad_a."""
        n, ldv = psi_n.shape[0], psi_n.shape[-1]
        an = np.ascontiguousarray(A_n, np.float64) if A_n is not None else None
        anp = np.ascontiguousarray(A_np1, np.float64) if A_np1 is not None else None
        ev = np.ascontiguousarray(e, np.float64) if e is not None else None
        ga = np.zeros(2) if want_grad_a else None
        _check(lib().qbg_etrs_adjoint_step(self.h, _dev_ptr(psi_n), ldv, n, None,
                                           float(dt), _np_ptr(an), _np_ptr(anp), _np_ptr(ev),
                                           _dev_ptr(lam), _dev_ptr(grad_v), _np_ptr(ga),
                                           _stream_ptr(stream)), "qbg_etrs_adjoint_step")
        return ga


class TDPropagation:
    """Checkpointed forward/backward operator pair over nsteps fixed-potential
    ETRS steps of one plan (qbg_td_*): forward() propagates psi in place
    under a per-step vector potential A[n] and returns the current J[n];
    backward(dLdJ) returns the gradients of a loss of the currents with
    respect to v(r) and to the vector potential along a direction e."""

    def __init__(self, H, psi, occ, dt, nsteps, K=20):
        self.H = H
        self.nst, self.ld = int(psi.shape[0]), int(psi.shape[-1])
        self.nsteps = int(nsteps)
        self._occ = np.ascontiguousarray(occ, np.float64)
        h = _P()
        _check(lib().qbg_td_create(H.h, self.ld, self.nst, _np_ptr(self._occ), float(dt),
                                   self.nsteps, int(K), ctypes.byref(h)), "qbg_td_create")
        self.h = h

    def forward(self, psi, A, stream=None):
        A = np.ascontiguousarray(np.broadcast_to(np.asarray(A, np.float64),
                                                 (self.nsteps + 1, 3)))
        J = np.zeros((self.nsteps + 1, 3))
        _check(lib().qbg_td_forward(self.h, _dev_ptr(psi), _np_ptr(A), _np_ptr(J),
                                    _stream_ptr(stream)), "qbg_td_forward")
        return J

    def backward(self, dLdJ, e=None, grad_v=None, lambda0=None, stream=None):
        """grad_v: device array of N doubles (overwritten) or None; returns
        dL/da_n along e (numpy, nsteps+1) when e is given, else None."""
        g = np.ascontiguousarray(dLdJ, np.float64).reshape(self.nsteps + 1, 3)
        ev = np.ascontiguousarray(e, np.float64) if e is not None else None
        ga = np.zeros(self.nsteps + 1) if e is not None else None
        _check(lib().qbg_td_backward(self.h, _np_ptr(g), _np_ptr(ev), _dev_ptr(grad_v),
                                     _np_ptr(ga), _dev_ptr(lambda0), _stream_ptr(stream)),
               "qbg_td_backward")
        return ga

    def close(self):
        if getattr(self, "h", None):
            lib().qbg_td_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def selftest_wait_timeout(polls=20000):
    """Run one bounded device wait that must expire; returns the status."""
    return int(lib().qbg_selftest_wait_timeout(int(polls)))


class EtrsGraph:
    """One ETRS step of many independent cells captured as one CUDA graph.

    cells: list of (Hamiltonian, psi device tensor [nst, ld], occ numpy).
    Each Hamiltonian must be a distinct plan; psi tensors stay owned by the
    caller and are advanced in place by every launch()."""

    def __init__(self, cells, dt, stream=None):
        n = len(cells)
        self.cells = cells
        self._plans = (_P * n)(*[c[0].h for c in cells])
        self._psi = (_P * n)(*[_dev_ptr(c[1]) for c in cells])
        self._ld = (ctypes.c_int * n)(*[int(c[1].shape[-1]) for c in cells])
        self._nst = (ctypes.c_int * n)(*[int(c[1].shape[0]) for c in cells])
        self._occ_arrays = [np.ascontiguousarray(c[2], np.float64) for c in cells]
        self._occ = (_P * n)(*[_np_ptr(o) for o in self._occ_arrays])
        g = _P()
        _check(lib().qbg_etrs_graph_create(n, self._plans, self._psi, self._ld, self._nst,
                                           self._occ, float(dt), _stream_ptr(stream),
                                           ctypes.byref(g)), "qbg_etrs_graph_create")
        self.h = g

    def launch(self, stream=None):
        _check(lib().qbg_etrs_graph_launch(self.h, _stream_ptr(stream)), "qbg_etrs_graph_launch")

    def check(self):
        _check(lib().qbg_etrs_graph_check(self.h), "qbg_etrs_graph_check")

    def close(self):
        if getattr(self, "h", None):
            lib().qbg_etrs_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
