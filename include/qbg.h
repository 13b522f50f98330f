/*
 * qbg.h -- C ABI of qball-gb300, a GB300 (sm_103a) implementation of
 * qball's Kohn-Sham Hamiltonian application and ETRS real-time propagation
 * step.
 *
 * The entry points mirror the reference's own operator surface; each
 * declaration cites the reference interface it replaces (paths relative to
 * the qball source tree).  Conventions, identical to the reference:
 *
 *  - Complex numbers are interleaved (re, im) pairs: double[2] for the FP64
 *    ("plain") precision, float[2] where a _f32 entry point says so.
 *  - A wavefunction block is column-major [ld x nst] complex; column n holds
 *    state n, row ig the coefficient of plane wave ig in the basis' rod order
 *    (Basis.cc:596-680): rods (h,k) in the order given, the G vectors of a
 *    rod contiguous with l ascending from rod_lmin.
 *  - Real-space grids are indexed f[i + np0*(j + np1*k)]
 *    (FourierTransform.h:170).
 *  - backward: f(r) = sum_G c(G) exp(+iG.r), unscaled.  forward:
 *    c(G) = (1/N) sum_r f(r) exp(-iG.r), N = np0*np1*np2
 *    (FourierTransform.h:147-152).
 *  - All array arguments of compute entry points are DEVICE pointers unless
 *    the parameter comment says "host".  Calls are asynchronous on the given
 *    CUDA stream (NULL = legacy default stream) unless they return a host
 *    scalar, in which case they synchronise that stream first.  Calls that
 *    run tensor-core GEMMs (qbg_hpsi, qbg_etrs_step and the adjoint in the
 *    forms that use them) also synchronise the given stream before they
 *    return: they read the GEMMs' error word on that stream, so a bounded
 *    wait that expired is reported by the call that ran it
 *    (QBG_ERR_TIMEOUT).
 *  - Every function returns a qbg_status; no C++ exception crosses the ABI.
 *    qbg_last_error() gives a message for the last failure on this thread.
 *  - A plan is thread-compatible, not thread-safe: one plan per stream at a
 *    time (the reference's FourierTransform is not reentrant either).
 */
#ifndef QBG_H
#define QBG_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  QBG_OK = 0,
  QBG_ERR_INVALID = 1,     /* bad argument or inconsistent sizes */
  QBG_ERR_NOMEM = 2,       /* device or host allocation failed */
  QBG_ERR_UNSUPPORTED = 3, /* grid length with an unsupported prime factor */
  QBG_ERR_CUDA = 4,        /* a CUDA runtime call failed */
  QBG_ERR_TIMEOUT = 5,     /* a bounded device-side wait expired */
  QBG_ERR_DIVERGED = 6,    /* norm / charge drift check failed */
  QBG_ERR_STATE = 7        /* call made before the plan was set up for it */
} qbg_status;

enum {
  QBG_PREC_FP64 = 0,        /* plain form: FP64 storage and FP64 arithmetic */
  QBG_PREC_MIXED = 1,       /* FP32 transforms, tensor-core projector GEMMs
                               (2-piece FP16 split), FP64 kinetic term, FP64
                               wavefunctions, Taylor sums and reductions */
  QBG_PREC_MIXED_FFT64 = 2, /* as MIXED but FP64 transforms */
  QBG_PREC_MIXED_NL64 = 3,  /* as MIXED but FP64 projector GEMMs */
  QBG_PREC_MIXED_DF32 = 4   /* as MIXED but double-float (FP32 pair)
                               transforms: ~48-bit, on the FP32 pipe; the
                               kinetic term and Taylor increment are
                               double-float products added to FP64 */
};

/* Projector GEMMs of the plain FP64 form (qbg_plan_set_fp64_gemm). */
enum {
  QBG_GEMM_SIMT = 0,  /* FP64 FMA on the CUDA cores */
  QBG_GEMM_OZAKI = 1  /* FP64-accurate on the tensor cores (the default): the
                         Ozaki scheme, operands split into 7-bit integer
                         slices (FP16, exact), slice products accumulated
                         exactly in FP32 tensor memory over windows of K */
};

typedef struct qbg_plan qbg_plan;

const char* qbg_last_error(void);
const char* qbg_version(void);

/* ---- Basis: Basis::resize (Basis.cc:302-700) -------------------------- */
/* Full-sphere (force_complex) basis at k=0 on one process, rods in the
 * reference's order.  a: host double[9] = cell vectors a0,a1,a2 (bohr);
 * ecut in Hartree (the reference stores ecut in Ha, Ecut.h:80).
 * info (host int[12]): [0]=ngw [1]=nrods [2..4]=np (Basis::np) [5..7]=idxmin
 * [8..10]=idxmax [11]=0.  qbg_basis_fill's outputs are host arrays of
 * nrods / nrods / nrods / nrods / 3*ngw / ngw / 3*ngw (any may be NULL);
 * kpgx is stored as x block, y block, z block (Basis::kpgx_ptr). */
qbg_status qbg_basis_dims(const double* a, double ecut, int* info);
qbg_status qbg_basis_fill(const double* a, double ecut, int* rod_h,
                          int* rod_k, int* rod_lmin, int* rod_size, int* idx,
                          double* kpg2, double* kpgx);

/* ---- Plan: FourierTransform(basis, np0, np1, np2)
 *            (FourierTransform.h:136, FourierTransform.cc:144-527) -------- */
typedef struct {
  int ngw;             /* Basis::localsize() */
  int nrods;           /* Basis::nrod_loc() */
  const int* rod_h;    /* host, nrods: Basis::rod_h */
  const int* rod_k;    /* host, nrods: Basis::rod_k */
  const int* rod_lmin; /* host, nrods: Basis::rod_lmin */
  const int* rod_size; /* host, nrods: Basis::rod_size */
  const double* kpgx;  /* host, 3*ngw: Basis::kpgx_ptr(0..2) */
  double omega;        /* UnitCell::volume() */
} qbg_basis_desc;

/* Descriptors are copied; nothing is borrowed past the call.  Fails with
 * QBG_ERR_UNSUPPORTED for grid lengths with prime factors other than
 * 2,3,5,7,11,13 and QBG_ERR_INVALID when a rod or band row falls outside
 * the grid (np0 <= 2*max|h|, np1 < 2*(max|k|+1) or np2 <= 2*max|l|). */
qbg_status qbg_plan_create(const qbg_basis_desc* basis, int np0, int np1,
                           int np2, int precision, qbg_plan** plan);
qbg_status qbg_plan_destroy(qbg_plan* plan);
/* states processed per transform launch group (L2 working-set control) */
qbg_status qbg_plan_set_chunk(qbg_plan* plan, int states_per_chunk);
/* How the plain FP64 form (precision QBG_PREC_FP64) runs the two complex
 * GEMMs of NonLocalPotential::energy (NonLocalPotential.cc:2064, 2165):
 * QBG_GEMM_OZAKI (default) on the tensor cores with every row scaled by a
 * power of two and written as `slices` balanced 7-bit digits (7: 49 bits,
 * 6: 42 bits; the digit products of equal weight summed exactly), or
 * QBG_GEMM_SIMT with FP64 FMAs.  Both match FP64 to rounding level of the
 * row maxima; the tensor-core form is ~70x faster on GB300, whose FP64 pipe
 * runs at 1/72 of FP32.  Other forms ignore the setting. */
qbg_status qbg_plan_set_fp64_gemm(qbg_plan* plan, int mode, int slices);

/* FourierTransform::backward(c, f) (FourierTransform.cc:529), batched over
 * nbatch states: c [ldc x nbatch] complex, f [N x nbatch] complex (FP64). */
qbg_status qbg_backward(qbg_plan* plan, const double* c, int ldc, double* f,
                        int nbatch, void* stream);
/* qbg_backward for callers that cannot allocate device memory at call time
 * (for example code being captured into a CUDA graph, where cudaMalloc
 * cannot be recorded, or a host application whose device memory is owned
 * by its own pool).  No counterpart in the reference.  Same arguments and
 * results as qbg_backward, but its scratch comes from one static 32 MiB
 * device array that the library holds on every GPU until exit instead of a
 * plan buffer, and it calls no cudaMalloc/cudaFree.  Limit: one state's
 * intermediates, 16*np2*(nrods + nband*np0) bytes with nband =
 * 2*(max|k|+1), must fit in 32 MiB, else QBG_ERR_INVALID.  The first call
 * on a device resolves the array's device address (make that first call
 * before any stream capture).  The address is kept for the life of the
 * process: no cudaDeviceReset of that device may come between calls.  Calls
 * share the array: two calls whose kernels overlap on the GPU race, so
 * serialise them (one stream).  The array needs no clearing (every element
 * read is first written by the same call). */
qbg_status qbg_backward_noalloc(qbg_plan* plan, const double* c, int ldc,
                                double* f, int nbatch, void* stream);

/* FourierTransform::forward(f, c) (FourierTransform.cc:542), batched; like
 * the reference, f is overwritten (used as scratch). */
qbg_status qbg_forward(qbg_plan* plan, double* f, double* c, int ldc,
                       int nbatch, void* stream);

/* ---- Hamiltonian set-up ---------------------------------------------- */
/* Local potential v(r) on the grid (EnergyFunctional::v_r,
 * EnergyFunctional.h:104).  v_r: N doubles, host or device (cudaMemcpy
 * with cudaMemcpyDefault). */
qbg_status qbg_set_vlocal(qbg_plan* plan, const double* v_r);

/* The FP64 local potential in use (EnergyFunctional::v_r, set by
 * qbg_set_vlocal or rebuilt by qbg_update_vhxc): N doubles to v_r, host or
 * device (cudaMemcpyDefault); synchronises the device. */
qbg_status qbg_get_vlocal(const qbg_plan* plan, double* v_r);

/* Kleinman-Bylander projectors of nsp species with the synthetic radial
 * form v_l(g) = g^l exp(-g^2 rc^2/2) (stands in for Species::dvnlg,
 * Species.cc:1492).  All host arrays: na[nsp], lmax[nsp] in {-1,0,1,2},
 * rc[nsp], wt[3*nsp] (KB weight per species and l, NonLocalPotential.cc:
 * 228-236), tau[3*sum(na)] atom positions (bohr).  Replaces
 * NonLocalPotential::init + update_twnl (NonLocalPotential.cc:76-259,
 * 261-760). */
qbg_status qbg_set_nonlocal(qbg_plan* plan, int nsp, const int* na,
                            const int* lmax, const double* rc,
                            const double* wt, const double* tau);

/* Kleinman-Bylander projectors given as tables, for real pseudopotentials:
 * the arrays NonLocalPotential::init and update_twnl build
 * (NonLocalPotential.cc:76-259, 261-760) from Species::dvnlg (Species.cc:
 * 1492) and the real harmonics.  All host arrays, species after species:
 * na[nsp] atoms and npr[nsp] projectors per species; lproj[sum npr] the
 * angular momentum (0..3) of projector ipr (NonLocalPotential::lproj);
 * wt[sum npr] its KB weight in Hartree (NonLocalPotential::wt, i.e.
 * Species::wsg); twnl[sum npr][ngw] its radial-angular factor on the basis
 * (twnl[is][ig + ngw*ipr]), evaluated at |k+G-A| for the vector potential in
 * force; tau[3*sum na] atom positions (bohr).  H then applies
 * anl = twnl (-i)^l exp(-i(k+G-A).tau) exactly as NonLocalPotential::energy
 * (:1962-2037).  The tables depend on A: after qbg_set_vector_potential the
 * caller passes them again for the new A, as the reference re-runs
 * update_twnl (EnergyFunctional.cc:2047-2055); the adjoint's derivative
 * along A is not available with tables (QBG_ERR_UNSUPPORTED).  Replaces
 * what qbg_set_nonlocal set. */
qbg_status qbg_set_nonlocal_tables(qbg_plan* plan, int nsp, const int* na,
                                   const int* npr, const int* lproj,
                                   const double* wt, const double* twnl,
                                   const double* tau);

/* Velocity-gauge vector potential A (host double[3]); recomputes
 * |k+G-A|^2 (VectorPotential::get_kpgpa2, VectorPotential.h:84-95) and the
 * projector tables for k+G-A (EnergyFunctional::vector_potential_changed,
 * EnergyFunctional.cc:2047-2055). */
qbg_status qbg_set_vector_potential(qbg_plan* plan, const double* A);

/* ---- Operators --------------------------------------------------------- */
/* hpsi = H psi for nst states: EnergyFunctional::energy(psi,
 * compute_hpsi=true, dwf, ...) (EnergyFunctional.cc:1128-1701): dwf cleared,
 * nonlocal projectors (NonLocalPotential::energy, NonLocalPotential.cc:
 * 1908-2170), kinetic 0.5|k+G-A|^2 c, then SlaterDet::rs_mul_add
 * (SlaterDet.cc:1025-1037).  psi, hpsi: [ld x nst] complex FP64.  occ: host
 * double[nst] or NULL; when enl (host double*) is non-NULL it receives the
 * nonlocal energy sum_n occ_n sum_p D_p/Omega |<beta_p|psi_n>|^2 and the
 * call synchronises the stream. */
qbg_status qbg_hpsi(qbg_plan* plan, const double* psi, int ld, double* hpsi,
                    int nst, const double* occ, double* enl, void* stream);

/* ChargeDensity::update_density (ChargeDensity.cc:276-556) without
 * symmetrisation or ultrasoft/NLCC terms: rho(r) = sum_n (weight occ_n /
 * Omega) |psi_n(r)|^2 (SlaterDet::compute_density, SlaterDet.cc:905-925).
 * rho: device double[N], overwritten.  nel (host, may be NULL) receives
 * Omega/N sum_r rho (ChargeDensity.cc:515-528) and synchronises. */
qbg_status qbg_density(qbg_plan* plan, const double* psi, int ld, int nst,
                       const double* occ, double weight, double* rho,
                       double* nel, void* stream);

/* Total electronic current J (host double[3]) of CurrentDensity::
 * update_current (CurrentDensity.cc:39-106), evaluated in G space:
 * J_d = -sum_n occ_n sum_G (k+G)_d |c_nG|^2 + A_d nel.  Synchronises. */
qbg_status qbg_current(qbg_plan* plan, const double* psi, int ld, int nst,
                       const double* occ, double nel, double* J,
                       void* stream);

/* ---- Hartree + exchange-correlation potential -------------------------- */
/* Density basis of ChargeDensity (ChargeDensity.cc:76-100: the sphere
 * |G|^2/2 < ecutden, 4 ecut by default) on the plan's grid, for the
 * transforms of the density and of the local potential (vft).  The basis
 * must fit the plan's np0 x np1 x np2 grid (FourierTransform.cc:150-200);
 * the descriptor's kpgx are the G vectors (k = 0). */
qbg_status qbg_set_density_basis(qbg_plan* plan, const qbg_basis_desc* vbasis);

/* Ionic terms on the density basis: vion_local_g and rhopst of
 * EnergyFunctional (EnergyFunctional.cc:1895-1915: species' local
 * pseudopotentials and Gaussian pseudo-charges times structure factors).
 * Host complex double[2*ngv] each, in the density basis' order; rhopst_g may
 * be NULL (zero). */
qbg_status qbg_set_ionic_terms(qbg_plan* plan, const double* vion_g,
                               const double* rhopst_g);

/* Fourier coefficients of the charge, rhog = forward_v(Omega rho(r))
 * (ChargeDensity.cc:515-550).  rho: device double[N]; rhog: device complex
 * double[2*ngv]. */
qbg_status qbg_density_g(qbg_plan* plan, const double* rho, double* rhog,
                         void* stream);

/* EnergyFunctional::update_hamiltonian + update_vhxc (EnergyFunctional.cc:
 * 300-520, TD branch) with the LDA functional (XCPotential::update,
 * XCPotential.cc:130-190; LDAFunctional::xc_unpolarized, LDAFunctional.cc:
 * 102-160): from rho (device double[N]) the local potential becomes
 *   v_r = vxc(rho) + Re backward_v(vion_g + 4 pi (rho_G + rhopst_G) / |G|^2)
 * with rho_G = forward_v(rho); it replaces what qbg_set_vlocal set.  en
 * (host double[3], may be NULL) receives {E_H, E_xc, E_ps} (ehart_, exc_,
 * eps_) and the call then synchronises. */
qbg_status qbg_update_vhxc(qbg_plan* plan, const double* rho, double* en,
                           void* stream);

/* on != 0: qbg_etrs_step rebuilds v_r by qbg_update_vhxc from the density of
 * psi(t) before preupdate (loop top of EhrenSampleStepper::step,
 * EhrenSampleStepper.cc:322-329) and from the density of the predicted
 * psi(t+dt) in update() (ExponentialWavefunctionStepper.cc:259-261).  Needs
 * qbg_set_density_basis and qbg_set_ionic_terms first. */
qbg_status qbg_set_selfconsistent(qbg_plan* plan, int on);

/* on != 0: approximated ETRS, the stepper's AETRS option (ExponentialWave-
 * functionStepper with approximated_, ExponentialWavefunctionStepper.cc:
 * 153-276; SelfConsistentPotential::extrapolate, SelfConsistentPotential.cc:
 * 46-73).  Every qbg_etrs_step stores the local potential of H(t) (after the
 * self-consistent rebuild when that is on); from the third stored step on,
 * psi(t) is propagated half a step with H(t), then half a step with the
 * potential extrapolated as 3 v(t) - 3 v(t-dt) + v(t-2dt) and the vector
 * potential A_t (the reference's preupdate runs before the vector potential
 * moves on), and no predicted state or density is formed: 8 H|psi> per step
 * instead of 12, and one density (the loop top's) instead of two.  rho_mid and
 * nel then receive the density of psi(t+dt).  Switching resets the stored
 * potentials. */
qbg_status qbg_set_aetrs(qbg_plan* plan, int on);

/* SlaterDet::gram (SlaterDet.cc:1043-1143, complex branch, norm-conserving):
 * psi [ld x nst] FP64 is orthonormalised in place, C <- C L^{-H} with
 * C^H C = L L^H.  The overlap C^H C and the product with L^{-H} (2 x 8 nst^2
 * ngw flop) run on the device in FP64; the nst x nst Cholesky factor and its
 * inverse are formed on the host.  QBG_ERR_DIVERGED when the overlap is not
 * positive definite.  Synchronises the stream. */
qbg_status qbg_gram(qbg_plan* plan, double* psi, int ld, int nst, void* stream);

/* One ETRS step (ExponentialWavefunctionStepper::preupdate + update,
 * ExponentialWavefunctionStepper.cc:153-276; 4th-order Taylor
 * exponentials, ExponentialWavefunctionStepper.cc:51-148): psi [ld x nst]
 * FP64 is advanced in place from t to t+dt.  A_t (host double[3]) is the
 * vector potential for the two exponentials of preupdate, A_tdt for the
 * exponential of update (EhrenSampleStepper.cc:477-548); NULL means
 * "unchanged".  rho_mid (device double[N], may be NULL) receives the density
 * of the predicted psi(t+dt) built inside update() (ExponentialWavefunction-
 * Stepper.cc:259); nel (host, may be NULL) its electron count.  With a
 * reduced-precision form the three exponentials apply H in that form and
 * accumulate the Taylor series into the FP64 psi.  After
 * qbg_set_selfconsistent(plan, 1) the local potential is rebuilt from the
 * density of psi(t) before preupdate and from rho_mid before update. */
qbg_status qbg_etrs_step(qbg_plan* plan, double* psi, int ld, int nst,
                         const double* occ, double dt, const double* A_t,
                         const double* A_tdt, double* rho_mid, double* nel,
                         void* stream);

/* ---- Adjoint of the ETRS step (no reference counterpart: the reference
 *      propagates forward only; the step differentiated is that of
 *      ExponentialWavefunctionStepper.cc:153-276 with a fixed local
 *      potential, i.e. qbg_etrs_step without qbg_set_selfconsistent) ----- */
/* One step psi_{n+1} = P(H(A_{n+1})) P(H(A_n)) psi_n, P = 4th-order Taylor
 * polynomial of exp(-i H dt/2), taken backwards.  With the adjoint state
 * lambda defined by dL = 2 Re sum_s <lambda_s|d psi_s>:
 *   lambda (device [ld x nst], in: lambda_{n+1}) <- P_a^+ P_b^+ lambda;
 *   grad_v (device double[N], may be NULL) += dL/dv(r) of the plan's local
 *     potential on the grid points, through this step;
 *   grad_a (host double[2], may be NULL) += dL/da_n, dL/da_{n+1}: the
 *     derivatives along the unit direction e (host double[3]) of the vector
 *     potential, through the kinetic term |k+G-A|^2/2 and the projectors
 *     beta(k+G-A) (NonLocalPotential.cc:1962-2037).
 * psi_n: device state at t_n (not modified).  A_n, A_np1: host double[3] or
 * NULL (keep the plan's A); the plan is left at A_n.  occ is not used
 * (reserved).  Runs the forward of the step again (8 H applications,
 * keeping the Taylor powers and their projections), then 8 H applications,
 * 16 backward transforms and, with grad_a, 16 projections on the derivative
 * of the projector table along e.  Synchronises when grad_a is given. */
qbg_status qbg_etrs_adjoint_step(qbg_plan* plan, const double* psi_n, int ld,
                                 int nst, const double* occ, double dt,
                                 const double* A_n, const double* A_np1,
                                 const double* e, double* lambda,
                                 double* grad_v, double* grad_a, void* stream);

/* Checkpointed forward/backward operator pair over nsteps fixed-potential
 * ETRS steps (nsteps >= 1) with a per-step vector potential (laser field in
 * the velocity gauge, VectorPotential.h:150-160).  The forward pass keeps
 * psi every K steps in device memory (ceil(nsteps/K) copies); the backward
 * pass recomputes each segment of K steps from its checkpoint, keeping per
 * step psi_n, the half step, the Taylor powers H^1..3 of both and their
 * projections (8 state-sized buffers per step, 8K in all), and runs the
 * adjoint steps in reverse: 16 H applications per step in all.  The
 * operator pair borrows the plan (which must outlive it, as Basis must
 * outlive FourierTransform in the reference) and uses the plan's stream
 * rules: one operator pair or plan call at a time per plan. */
typedef struct qbg_td qbg_td;
qbg_status qbg_td_create(qbg_plan* plan, int ld, int nst, const double* occ,
                         double dt, int nsteps, int K, qbg_td** td);
/* psi (device [ld x nst]): psi_0 in, psi_nsteps out.  A: host double
 * [(nsteps+1) x 3], A_n at t_n.  J (host double[(nsteps+1) x 3] or NULL):
 * the total current of every psi_n at A_n, as qbg_current with nel = sum occ.
 * Synchronises. */
qbg_status qbg_td_forward(qbg_td* td, double* psi, const double* A, double* J,
                          void* stream);
/* Gradients of a loss L(J_0..J_nsteps) given dLdJ (host double[(nsteps+1)
 * x 3]): grad_v (device double[N] or NULL) = dL/dv(r); grad_a (host double
 * [nsteps+1] or NULL) = dL/da_n along e (host double[3], required with
 * grad_a), including the explicit A_n nel term of J_n; lambda0 (device
 * [ld x nst] or NULL) = the adjoint state of psi_0.  Needs a forward pass.
 * Synchronises. */
qbg_status qbg_td_backward(qbg_td* td, const double* dLdJ, const double* e,
                           double* grad_v, double* grad_a, double* lambda0,
                           void* stream);
qbg_status qbg_td_destroy(qbg_td* td);

/* ---- Batched cells as one CUDA graph (no reference counterpart: the
 *      reference steps one system per process group) -------------------- */
typedef struct qbg_graph qbg_graph;
/* Capture one ETRS step (qbg_etrs_step with A unchanged, no rho_mid/nel) of
 * each of ncells independent cells -- distinct plans of any grid, basis, form
 * and state count, psi[i] [ld[i] x nst[i]] with host occupations occ[i] --
 * into one CUDA graph whose cells run as concurrent branches.  One
 * uncaptured step runs first on scratch copies of the states (psi is not
 * changed) so that the capture allocates and synchronises nothing; the
 * occupations and vector potentials in force then must stay unchanged while
 * the graph is used.  stream may be NULL (an internal stream captures). */
qbg_status qbg_etrs_graph_create(int ncells, qbg_plan* const* plans,
                                 double* const* psi, const int* ld,
                                 const int* nst, const double* const* occ,
                                 double dt, void* stream, qbg_graph** graph);
/* one ETRS step of every cell (asynchronous on stream) */
qbg_status qbg_etrs_graph_launch(qbg_graph* graph, void* stream);
/* synchronise the device and read every cell's tensor-core status word
 * (QBG_ERR_TIMEOUT if a bounded wait expired during a replay) */
qbg_status qbg_etrs_graph_check(qbg_graph* graph);
qbg_status qbg_etrs_graph_destroy(qbg_graph* graph);

/* Autotuner: time H|psi> (two applications after a warm-up) over the
 * plan's transform shapes -- radix order of the Stockham passes (0: 8/4/2
 * first, 1: odd primes first, 2: radix 4 preferred), prime-factor in-place
 * splits on/off, the fused x-y-x kernel (whole-plane, band-row, off), the
 * register lane-group y pass on/off (FP32 transforms) -- then over states
 * per transform launch group in {8, 16, 32, 64, 96, 144}, and keep the
 * fastest for this plan; *chosen (may be NULL) receives the states per
 * group.  Synchronises. */
qbg_status qbg_plan_autotune(qbg_plan* plan, const double* psi, int ld, int nst,
                             const double* occ, void* stream, int* chosen);

/* Transform shape of a plan (what qbg_plan_autotune searches; every shape
 * gives the same results to rounding): radix_order 0..2 as above,
 * prime_factor / lane_group 0 or 1, fused 0 (separate x, y, x kernels),
 * 1 (band-row fused kernel) or 2 (whole-plane kernel on 120 x 120 planes,
 * the default; other planes run as 1).  Synchronises when the radix order
 * changes (the tables are rebuilt). */
qbg_status qbg_plan_set_transform_config(qbg_plan* plan, int radix_order,
                                         int prime_factor, int fused,
                                         int lane_group);
/* cfg (host int[5]): states per group, radix order, prime-factor splits,
 * fused x-y-x kernel (0..2), lane-group y pass. */
qbg_status qbg_plan_get_transform_config(const qbg_plan* plan, int* cfg);

/* Diagnostic, no reference counterpart: runs one bounded mbarrier wait that
 * nothing completes (polls polls, 1..2^20) and returns QBG_ERR_TIMEOUT when
 * it gives up as designed -- the path every wait of the tensor-core kernel
 * takes instead of hanging.  The device stays usable.  Synchronises. */
qbg_status qbg_selftest_wait_timeout(int polls);

/* Diagnostic, no reference counterpart: poll limit of the pipeline waits of
 * this plan's tensor-core GEMMs (-1 restores the default, ~0.2 s; 0 makes
 * every such wait give up at once).  The waits for a CTA's own copies and
 * MMAs to land before it frees its memory keep the default limit, so an
 * expired wait ends the launch cleanly: the call that ran it returns
 * QBG_ERR_TIMEOUT and the plan stays usable.  For tests of that path. */
qbg_status qbg_plan_set_wait_polls(qbg_plan* plan, int polls);

/* ---- Instrumentation (no reference counterpart beyond its TimerMap,
 *      NonLocalPotential.cc:54, EhrenSampleStepper.cc:1136-1149) ------- */
/* Number of this library's kernel launches issued since plan creation. */
qbg_status qbg_launch_count(const qbg_plan* plan, long long* count);
/* enable != 0: bracket every kernel launch with CUDA events on its stream
 * and accumulate per-phase device time (each launch then runs alone); the
 * accumulators are reset by every call. */
qbg_status qbg_profile(qbg_plan* plan, int enable);
/* ms[i], launches[i] for phases i < n (qbg_phase_name(i) gives the name;
 * there are 13 phases). */
qbg_status qbg_profile_read(const qbg_plan* plan, double* ms,
                            long long* launches, int n);
const char* qbg_phase_name(int phase);

#ifdef __cplusplus
}
#endif
#endif /* QBG_H */
