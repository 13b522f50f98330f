/* qbo.h -- CPU oracle for the qball H|psi> / ETRS hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C FP64 restatement of the
 * reference's algorithms, used by tests/ as the parity checker and by
 * bench.py as the timed CPU baseline.  The product (libqbg.so) never links,
 * loads or calls it.  Every function cites the reference file:line it
 * restates (paths relative to the qball source tree).
 *
 * Parity pinning: the basis builder and the 3D transform are checked
 * bit-for-bit against the reference's own Basis.cc / FourierTransform.cc
 * (compiled into oracle/_ref by oracle/build_ref.sh, golden vectors committed
 * in tests/golden/).  The operator restatements above the transform
 * (rs_mul_add, the kinetic term, the nonlocal projectors, the density, the
 * current and the ETRS propagator) have no compiled reference counterpart
 * here (their sources need MPI/BLACS/ScaLAPACK/BLAS); they are pinned through
 * the transform plus independent identities checked in tests/.
 *
 * Complex arrays are interleaved (re, im) doubles.  Wavefunction blocks are
 * column-major [ld x nst] complex, G in the basis' rod order.
 */
#ifndef QBG_ORACLE_QBO_H
#define QBG_ORACLE_QBO_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Basis (Basis.cc:302-700, complex full-sphere branch, one process) ---- */
/* info: [0]=size(ngw) [1]=nrods [2..4]=np [5..7]=idxmin [8..10]=idxmax */
int qbo_basis_dims(const double* a, double ecut, int* info);
void qbo_basis_fill(const double* a, double ecut, int* rod_h, int* rod_k,
                    int* rod_lmin, int* rod_size, int* idx, double* kpg2,
                    double* kpgx);
double qbo_cell_volume(const double* a);
void qbo_cell_b(const double* a, double* b);
int qbo_factorizable(int n);

/* ---- FourierTransform (FourierTransform.cc:144-527, 529-583, FFT_NOLIB) ---- */
typedef struct qbo_ft qbo_ft;
qbo_ft* qbo_ft_create(int ngw, int nrods, const int* rod_h, const int* rod_k,
                      const int* rod_lmin, const int* rod_size, int np0,
                      int np1, int np2, int ntrans0);
void qbo_ft_destroy(qbo_ft* ft);
void qbo_ft_backward(const qbo_ft* ft, const double* c, double* f);
void qbo_ft_forward(const qbo_ft* ft, double* f, double* c);
void qbo_cfftm(double* ain, double* aout, double scale, int ntrans,
               int length, int ainc, int ajmp, int idir);

/* ---- Hamiltonian context ---- */
typedef struct qbo_ham qbo_ham;
/* kpgx: 3*ngw (x block, y block, z block) of k+G, no vector potential.
 * v_r: np012 doubles (copied).  One projector species set:
 *   nsp species; species s has na[s] atoms at tau[3*(first atom)..],
 *   lmax[s] in {-1 (local only),0,1,2}, rc[s] (synthetic KB radial
 *   v_l(g)=g^l exp(-g^2 rc^2/2)), wt[s*3+l] the KB weight D_l (Ha). */
qbo_ham* qbo_ham_create(const qbo_ft* ft, int ngw, const double* kpgx,
                        double omega, const double* v_r, int nsp,
                        const int* na, const int* lmax, const double* rc,
                        const double* wt, const double* tau);
void qbo_ham_destroy(qbo_ham* h);
/* Vector potential A (velocity gauge); recomputes |k+G-A|^2 and twnl
 * (VectorPotential.h:84-120, NonLocalPotential.cc:261-760). */
void qbo_ham_set_A(qbo_ham* h, const double* A);
int qbo_ham_nproj(const qbo_ham* h);
/* twnl for projector p (after set_A), ngw doubles; lproj / wt per projector */
void qbo_ham_set_species_tables(qbo_ham* h, int s, int npr, const int* lproj,
                                const double* wt, const double* twnl);
void qbo_ham_projector(const qbo_ham* h, int p, double* twnl, int* l,
                       double* wt, double* tau3);
/* cp = H c for nst states (EnergyFunctional.cc:1142-1152,1500,1639-1701);
 * returns E_nl (NonLocalPotential.cc:2124-2146) with occupations occ. */
double qbo_hpsi(const qbo_ham* h, const double* c, int ld, int nst,
                const double* occ, double* cp, int nthreads);
/* individual pieces, accumulating into cp */
double qbo_nl_apply(const qbo_ham* h, const double* c, int ld, int nst,
                    const double* occ, double* cp, int nthreads);
void qbo_kinetic_add(const qbo_ham* h, const double* c, int ld, int nst,
                     double* cp);
void qbo_rs_mul_add(const qbo_ham* h, const double* c, int ld, int nst,
                    double* cp, int nthreads);

/* rho += sum_n (weight*occ_n/omega) |bwd(c_n)|^2 (SlaterDet.cc:905-925) */
void qbo_compute_density(const qbo_ft* ft, const double* c, int ld, int nst,
                         const double* occ, double weight, double omega,
                         double* rho, int nthreads);
/* ChargeDensity::update_density (ChargeDensity.cc:276-556), nsym=0, NC:
 * rho zeroed then filled; returns the electron count Omega/N sum(rho). */
double qbo_update_density(const qbo_ft* ft, const double* c, int ld, int nst,
                          const double* occ, double omega, double* rho,
                          int nthreads);
/* total electronic current (CurrentDensity.cc:39-106), real-space route */
void qbo_current_rs(const qbo_ft* ft, const double* kpgx, int ngw,
                    const double* c, int ld, int nst, const double* occ,
                    double omega, const double* A, double nel, double* J,
                    int nthreads);
/* same quantity by Parseval in G space */
void qbo_current_g(const double* kpgx, int ngw, const double* c, int ld,
                   int nst, const double* occ, const double* A, double nel,
                   double* J);

/* Hartree + LDA update of the local potential (EnergyFunctional::
 * update_vhxc, EnergyFunctional.cc:353-520, TD branch; LDA of
 * LDAFunctional::xc_unpolarized, functionals/LDAFunctional.cc:102-160):
 *   rho_G = forward_v(omega rho(r)) / omega on the density basis
 *           (ChargeDensity.cc:515-550, EnergyFunctional.cc:300-323),
 *   v_r = vxc(rho(r)) + Re backward_v(vion_g + 4 pi (rho_G + rhopst_G) g2i).
 * vft: transform on the density basis (same grid); g2: its |G|^2 (ngv);
 * vion_g, rhopst_g: complex [ngv] (rhopst_g may be NULL = zero).
 * en (may be NULL) receives {E_H, E_xc, E_ps} (ehart_, exc_, eps_). */
double qbo_update_vhxc(const qbo_ft* vft, const double* g2, int ngv,
                       const double* vion_g, const double* rhopst_g,
                       const double* rho, double omega, double* v_r, double* en);
/* Fourier coefficients of the charge, rhog = forward_v(omega rho(r))
 * (ChargeDensity.cc:515-550); rhog complex [ngv]. */
void qbo_density_g(const qbo_ft* vft, const double* rho, double omega, double* rhog);
void qbo_lda(double rho, double* exc, double* vxc);

/* ETRS step (ExponentialWavefunctionStepper.cc:51-276, order 4, no Hxc
 * feedback): psi advanced in place from t to t+dt.  A_t applies to the
 * first two exponentials, A_tdt to the last one (EhrenSampleStepper.cc:
 * 477-548).  rho_mid (np012, may be NULL) receives the density of the
 * predicted psi(t+dt) formed inside update(); returns its electron count. */
double qbo_etrs_step(qbo_ham* h, double* psi, int ld, int nst,
                     const double* occ, double dt, const double* A_t,
                     const double* A_tdt, double* rho_mid, int nthreads);

/* The same step with the self-consistent Hamiltonian: v_r is rebuilt by
 * qbo_update_vhxc from the density of psi(t) before preupdate (the loop top
 * of EhrenSampleStepper::step, EhrenSampleStepper.cc:323-329) and from the
 * density of the predicted psi(t+dt) inside update()
 * (ExponentialWavefunctionStepper.cc:259-261). */
double qbo_etrs_step_hxc(qbo_ham* h, double* psi, int ld, int nst,
                         const double* occ, double dt, const double* A_t,
                         const double* A_tdt, const qbo_ft* vft,
                         const double* g2, int ngv, const double* vion_g,
                         const double* rhopst_g, double* rho_mid, int nthreads);

void qbo_ham_get_vr(const qbo_ham* h, double* v);
double qbo_aetrs_step(qbo_ham* h, double* psi, int ld, int nst, const double* occ,
                      double dt, const double* A_t, const double* A_tdt,
                      const qbo_ft* vft, const double* g2, int ngv,
                      const double* vion_g, const double* rhopst_g, double* vhist,
                      int* stored, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
