// qbg_internal.h -- plan layout and internal launchers shared by the .cu files.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/qbg.h"
#include "qbg_fft_engine.cuh"

namespace qbg {

void set_error(const char* fmt, ...);
qbg_status cuda_status(cudaError_t e, const char* what);

#define QBG_CUDA(call)                                              \
  do {                                                              \
    cudaError_t e_ = (call);                                        \
    if (e_ != cudaSuccess) return ::qbg::cuda_status(e_, #call);    \
  } while (0)

#define QBG_LAUNCHED(plan)                                          \
  do {                                                              \
    (plan)->launches++;                                             \
    cudaError_t e_ = cudaGetLastError();                            \
    if (e_ != cudaSuccess) return ::qbg::cuda_status(e_, "kernel"); \
  } while (0)

// Host-side factorisation and twiddle tables of one transform length.
struct LenTables {
  int n = 0;
  int npass = 0;
  int radix[kMaxPass] = {0};
  int ns[kMaxPass] = {0};
  int twoff[kMaxPass] = {0};
  int goff7 = 0, goff11 = 0, goff13 = 0;
  int ntw = 0;
  double2* d_tw64 = nullptr;
  double2* d_g64 = nullptr;
  float2* d_tw32 = nullptr;
  float2* d_g32 = nullptr;
  df32c* d_twdf = nullptr;
  df32c* d_gdf = nullptr;
  double2* d_root64 = nullptr;  // exp(-2 pi i m / n), m < n
  float2* d_root32 = nullptr;
  df32c* d_rootdf = nullptr;
  bool allow_pfa = true;  // prime-factor in-place split where the length has one
  template <typename T> FFTLen<T> view() const;
};

// Timed phases (names follow the reference's TimerMap keys where one exists:
// "fnl_gemm", "enl_hpsi" in NonLocalPotential.cc:2059-2170).
enum Phase {
  PH_FNL_GEMM = 0, PH_FNL_REDUCE, PH_ENL_HPSI, PH_Z_BWD, PH_X_BWD, PH_Y_VLOC,
  PH_X_FWD, PH_Z_FWD, PH_Y_DENSITY, PH_Y_STORE, PH_Y_LOAD, PH_MISC, PH_XYX_VLOC, PH_XY_PAIR,
  PH_COUNT
};
extern const char* const kPhaseName[PH_COUNT];

// Per-rod table entry: G offset of the rod's first coefficient, rod length,
// lmin, grid x index, band row index.
struct RodInfo {
  int first, size, lmin, xb;  // xb = x | (band << 16)
};

}  // namespace qbg

struct qbg_plan {
  int prec = QBG_PREC_FP64;
  int ngw = 0, nrods = 0;
  int np0 = 0, np1 = 0, np2 = 0;
  long long N = 0;
  int ntrans0 = 0, nband = 0;
  double omega = 0.0;
  double A[3] = {0, 0, 0};
  int chunk = 8;
  long long launches = 0;

  // transform tables (n0 along x, n1 along y, n2 along z)
  qbg::LenTables len[3];

  // device basis tables
  qbg::RodInfo* d_rods = nullptr;    // [nrods]
  int* d_row_ptr = nullptr;          // [nband+1] rods per band row (CSR)
  int* d_row_rod = nullptr;          // [nrods]
  int* d_row_x = nullptr;            // [nrods]
  int* d_band_y = nullptr;           // [nband] band row -> grid y
  double* d_kpgx = nullptr;          // [3*ngw] k+G
  double* d_kpg2A = nullptr;         // [ngw] |k+G-A|^2
  float* d_kpg2A32 = nullptr;        // [ngw]
  double* d_vr = nullptr;            // [N]
  float* d_vr32 = nullptr;           // [N]
  qbg::df32* d_vrdf = nullptr;       // [N]
  bool have_vr = false;
  std::vector<int> rod_h, rod_k, rod_lmin, rod_size;
  std::vector<double> kpgx_host;

  // nonlocal projectors
  int nproj = 0;
  int nsp = 0;
  std::vector<int> sp_na, sp_lmax;
  std::vector<double> sp_rc, sp_wt, sp_tau;
  bool nl_tables = false;      // projector tables given by the caller
  std::vector<int> sp_npr, sp_lproj;  // per species / per table row
  std::vector<double> sp_wtp;  // per table row: KB weight
  double* d_twnl = nullptr;    // [rows][ngw] the caller's twnl tables
  size_t twnl_bytes = 0;
  int* d_plist = nullptr;      // [nproj] packed (species, ipr, atom) -> int4-like
  double* d_ptau = nullptr;    // [3*nproj]
  double* d_pwt = nullptr;     // [nproj] wt/omega
  int* d_pl = nullptr;         // [nproj] (lm code)
  double* d_prc = nullptr;     // [nproj]
  double2* d_anl = nullptr;    // [nproj][ngw] FP64 projector table
  size_t anl_elems = 0;        // nproj * ngw of d_anl
  long long nl_version = 0;    // incremented by every table build
  void* d_pdesc = nullptr;     // [nproj] projector descriptors (qbg_nl.cu)
  void* d_adesc = nullptr;     // [nl_natoms] atom descriptors (qbg_nl.cu)
  int nl_natoms = 0;
  float2* d_anl32 = nullptr;   // [nproj][ngw] FP32 copy (mixed)
  bool nl_ready = false;
  void* tc = nullptr;          // tensor-core projector tables (mixed)
  void* oz = nullptr;          // FP64-accurate tensor-core projector tables (plain form)
  int fp64_gemm = QBG_GEMM_OZAKI;  // projector GEMMs of the plain FP64 form
  int oz_slices = 7;           // 7-bit slices per operand of those GEMMs (6 or 7)
  bool check_every_step = true; // read the tensor-core status word after each step
  int tc_polls = -1;            // poll limit of the GEMM pipeline waits (-1: default)
  bool lane_fft = true;         // register-resident lane-group transforms where supported
  bool fuse_xyx = true;         // x, y and x passes of H psi in one kernel where they fit
  bool plane_xyx = true;        // ... as the whole-plane kernel on 120 x 120 planes
  int nsm = 0;                  // SMs of the plan's device (set on first use)
  // adjoint pairing context, set around one H application (whole planes):
  // grad[r] += pair_scale * sum_s Re(conj(bwd psi_s(r)) G_s(r)), G [nst][N]
  // in the transform type, pair_slots one chunk of per-state slots
  const void* pair_G = nullptr;
  void* pair_slots = nullptr;
  double* pair_grad = nullptr;
  double pair_scale = 0.0;
  int radix_order = 0;          // Stockham radix order of the length tables (factorize)

  // scratch (allocated lazily, grown as needed)
  void* d_Z = nullptr;  size_t Z_bytes = 0;   // [chunk][n2][nrods]
  void* d_Y = nullptr;  size_t Y_bytes = 0;   // [chunk][n2][nband][n0]
  void* d_fnl = nullptr; size_t fnl_bytes = 0;       // [nst][nproj]
  void* d_fpart = nullptr; size_t fpart_bytes = 0;   // split-K partials
  double* d_red = nullptr; size_t red_bytes = 0;     // reduction partials
  double* d_rho = nullptr; size_t rho_bytes = 0;     // ETRS density scratch
  double* d_rho_slots = nullptr; size_t rho_slots_bytes = 0;  // [chunk][N] per-state density
  void* d_vsph = nullptr; size_t vsph_bytes = 0;      // [chunk][ngw] forward transform (sphere)
  double* h_red = nullptr; size_t h_red_bytes = 0;   // pinned host copy
  // phase profiler (off unless qbg_profile(plan, 1))
  bool prof = false;
  double prof_ms[qbg::PH_COUNT] = {0};
  long long prof_n[qbg::PH_COUNT] = {0};
  std::vector<double> occ_cache;  // last per-state factors uploaded to d_w[3]
  // ETRS work buffers
  void* d_w[4] = {nullptr, nullptr, nullptr, nullptr};
  size_t w_bytes[4] = {0, 0, 0, 0};
  // Hartree + xc update (qbg_hxc.cu)
  qbg_plan* vplan = nullptr;     // transform on the density basis, same grid
  double* d_g2i = nullptr;       // [ngv] 1/|G|^2 (0 at G = 0)
  double2* d_vion = nullptr;     // [ngv] vion_local_g
  double2* d_rhopst = nullptr;   // [ngv] rhopst (null: zero)
  double2* d_vg = nullptr;       // [ngv] rho_G, then v_G
  double2* d_vf = nullptr;       // [N] complex grid
  double* d_hxc_red = nullptr;   // energy partials [3][kHxcBlocks]
  bool have_ionic = false;
  bool selfconsistent = false;
  bool aetrs = false;            // approximated ETRS (qbg_set_aetrs)
  int aetrs_stored = 0;          // potentials stored so far (capped at 3)
  double* d_vhist = nullptr;     // [3][N] v_r at the top of the last three steps
  size_t vhist_bytes = 0;
  void* adj = nullptr;           // adjoint work buffers (qbg_adjoint.cu)
  double2* fnl_export = nullptr;  // when set: receives (D/Omega)<beta|psi> [nst][nproj] of
                                  // the next H application (device)
};

namespace qbg {

qbg_status ensure(void** p, size_t* cur, size_t need);

// Brackets one kernel launch with CUDA events when the plan's profiler is on
// (the stream is synchronised at the end of the bracket, so profiled runs
// measure each kernel alone).
struct PhaseTimer {
  qbg_plan* p;
  int ph;
  cudaStream_t st;
  cudaEvent_t a = nullptr, b = nullptr;
  PhaseTimer(qbg_plan* p_, int ph_, cudaStream_t st_) : p(p_), ph(ph_), st(st_) {
    if (p->prof) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, st);
    }
  }
  ~PhaseTimer() {
    if (p->prof) {
      cudaEventRecord(b, st);
      cudaEventSynchronize(b);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, a, b);
      p->prof_ms[ph] += ms;
      p->prof_n[ph] += 1;
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  }
};
qbg_status ensure_host(double** p, size_t* cur, size_t need);

// transforms (qbg_fft.cu); T = double or float.  Pointers are device.
// Hpsi local part for states [s0, s0+ns): out[g] = (out[g] + kin*psi[g]) +
// fwd(v * bwd(psi))[g] (out holds the nonlocal part, or zero when
// out_init == false); when acc != null: acc[g] += fac * out[g] (FP64).
// T is the arithmetic type of the transforms; wavefunctions, H psi and the
// accumulator are FP64 in memory.
template <typename T>
qbg_status local_hpsi(qbg_plan* p, const double2* psi, int ld, double2* out,
                      int nst, bool out_init, double2* acc, int ldacc,
                      double2 fac, cudaStream_t st);
template <typename T>
qbg_status backward(qbg_plan* p, const double2* c, int ldc, double2* f,
                    int nb, cudaStream_t st);
template <typename T>
qbg_status forward(qbg_plan* p, double2* f, double2* c, int ldc, int nb,
                   cudaStream_t st);
template <typename T>
qbg_status density(qbg_plan* p, const double2* c, int ldc, int nst,
                   const double* d_w, double* rho, cudaStream_t st);
// real-space fields F[s][z][y][x] = bwd(c_s)(r) in the transform type T on
// whole planes (120 x 120, FP64 or double-float transforms), F holding
// nst * N complex T values
template <typename T>
qbg_status plane_fields(qbg_plan* p, const double2* c, int ld, int nst, void* F, cudaStream_t st);

// whole-plane kernels (qbg_plane.cu): 120 x 120 planes, FP64 or
// double-float transforms, the plan's fused mode 2
bool plane_applies(const qbg_plan* p, bool fp32);
template <typename T> qbg_status plane_vloc(qbg_plan* p, int ns, int s0, cudaStream_t st);
template <typename T>
qbg_status plane_density(qbg_plan* p, int ns, const double* w, int acc, void* slots,
                         cudaStream_t st);
template <typename T> qbg_status plane_field(qbg_plan* p, int ns, double2* f, cudaStream_t st);
template <typename T>
qbg_status plane_fwd(qbg_plan* p, int ns, const double2* f, cudaStream_t st);
template <typename T> qbg_status plane_pair_field(qbg_plan* p, int ns, void* F, cudaStream_t st);

template <typename T>
qbg_status backward_scratch(qbg_plan* p, const double2* c, int ldc, double2* f, int nb,
                            void* Z, void* Y, int chunk, cudaStream_t st);

// nonlocal (qbg_nl.cu)
qbg_status nl_build(qbg_plan* p, cudaStream_t st);
template <typename T>
qbg_status nl_apply(qbg_plan* p, const cplx<T>* psi, int ld, cplx<T>* out,
                    int nst, const double* d_occ, double* enl_dev,
                    cudaStream_t st);

// tensor-core projector GEMMs (qbg_tc.cu): psi, out FP64 [ld x nst]
qbg_status tc_build(qbg_plan* p, cudaStream_t st);
void tc_release(qbg_plan* p);
void tc_invalidate(qbg_plan* p);  // the table changed; buffers kept
qbg_status tc_nl_apply(qbg_plan* p, const double2* psi, int ld, double2* out, int nst,
                       const double* d_occ, double* enl_part, int* enl_blocks,
                       cudaStream_t st);
qbg_status tc_check_status(qbg_plan* p, cudaStream_t st);

// FP64-accurate (Ozaki-scheme) tensor-core projector GEMMs (qbg_ozaki.cu)
qbg_status oz_build(qbg_plan* p, cudaStream_t st);
void oz_release(qbg_plan* p);
void oz_invalidate(qbg_plan* p);
qbg_status oz_nl_apply(qbg_plan* p, const double2* psi, int ld, double2* out, int nst,
                       const double* d_occ, double* enl_part, int* enl_blocks, cudaStream_t st);
qbg_status oz_check_status(qbg_plan* p, cudaStream_t st);

// misc kernels (qbg_ops.cu)
qbg_status update_kinetic(qbg_plan* p, cudaStream_t st);
// operator helpers (qbg_ops.cu)
qbg_status upload_occ(qbg_plan* p, const double* occ, int nst, double scale, double** d_out,
                      cudaStream_t st);
qbg_status hpsi_core(qbg_plan* p, const double2* psi, int ld, double2* out, int nst,
                     const double* d_occ, double* enl_part, int* enl_blocks, double2* acc,
                     int ldacc, double2 fac, cudaStream_t st);
bool uses_tc(const qbg_plan* p);
qbg_status check_common(qbg_plan* p, const void* a, int ld, int nst, const char* who);
qbg_status ensure_nl(qbg_plan* p, cudaStream_t st);
// psi <- sum_{k<=4} (-i dt1 H)^k / k! psi (FP64 accumulation)
qbg_status exponential(qbg_plan* p, double2* psi, int ld, int nst, const double* d_occ,
                       double dt1, cudaStream_t st);

// Gram orthonormalisation products (qbg_nl.cu), FP64 on the device
qbg_status gram_overlap(qbg_plan* p, const double2* psi, int ld, int nst, double2* S,
                        cudaStream_t st);
qbg_status gram_apply(qbg_plan* p, const double2* psi, int ld, int nst, const double2* T,
                      double2* out, int ldo, cudaStream_t st);

// adjoint support (qbg_nl.cu, qbg_tc.cu)
qbg_status nl_build_da(qbg_plan* p, const double* e, double2* dbeta, cudaStream_t st);
qbg_status nl_project64(qbg_plan* p, const double2* table, const double2* x, int ld, int nst,
                        double2* f, cudaStream_t st);
qbg_status tc_proj_build(qbg_plan* p, const double2* table, void** out, cudaStream_t st);
void tc_proj_free(void* proj);
qbg_status tc_project(qbg_plan* p, const void* proj, const double2* x, int ld, int nst,
                      double2* f, cudaStream_t st);
qbg_status tc_project_multi(qbg_plan* p, const void* proj, const double2* const* xs, int nvec,
                            int ld, int nst, double2* f, cudaStream_t st);
void adj_release(qbg_plan* p);

// Hartree + xc (qbg_hxc.cu): v_r from rho (device), energies stay on the
// device until read
qbg_status vhxc_update(qbg_plan* p, const double* rho, cudaStream_t st);
void hxc_release(qbg_plan* p);

}  // namespace qbg
