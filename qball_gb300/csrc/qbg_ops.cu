// qbg_ops.cu -- operator entry points of the C ABI: transforms, H|psi>,
// density, current and the ETRS step.
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "qbg_internal.h"

namespace qbg {
int nl_reduce_blocks(const qbg_plan* p, int nst);

#define QBG_TRY(x)                \
  do {                            \
    qbg_status s_ = (x);          \
    if (s_ != QBG_OK) return s_;  \
  } while (0)

__global__ void k_cvt64to32(const double2* __restrict__ a, int lda, float2* __restrict__ b,
                            int ldb, int ngw) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = blockIdx.y;
  if (g >= ngw) return;
  const double2 v = a[(size_t)n * lda + g];
  b[(size_t)n * ldb + g] = make_float2((float)v.x, (float)v.y);
}

__global__ void k_cvt32to64(const float2* __restrict__ a, int lda, double2* __restrict__ b,
                            int ldb, int ngw) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = blockIdx.y;
  if (g >= ngw) return;
  const float2 v = a[(size_t)n * lda + g];
  b[(size_t)n * ldb + g] = make_double2((double)v.x, (double)v.y);
}

__global__ void k_copy_cols(const double2* __restrict__ a, int lda, double2* __restrict__ b,
                            int ldb, int ngw) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = blockIdx.y;
  if (g >= ngw) return;
  b[(size_t)n * ldb + g] = a[(size_t)n * lda + g];
}

// per-block partial sums of x[i] (deterministic tree)
__global__ void k_sum(const double* __restrict__ x, long long n, double* __restrict__ part) {
  __shared__ double red[256];
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    s += x[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// current partials: part[3*(blockIdx.y*gridDim.x + blockIdx.x) + d] =
//   occ_n sum_{g in block} kpgx_d[g] |c_ng|^2
__global__ void k_current(const double2* __restrict__ c, int ld, int ngw,
                          const double* __restrict__ kpgx, const double* __restrict__ occ,
                          double* __restrict__ part) {
  __shared__ double red[3][256];
  const int n = blockIdx.y;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ngw; g += gridDim.x * blockDim.x) {
    const double2 v = c[(size_t)n * ld + g];
    const double a = v.x * v.x + v.y * v.y;
    s0 += kpgx[g] * a;
    s1 += kpgx[ngw + g] * a;
    s2 += kpgx[2 * ngw + g] * a;
  }
  red[0][threadIdx.x] = s0;
  red[1][threadIdx.x] = s1;
  red[2][threadIdx.x] = s2;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if (threadIdx.x < k)
      for (int d = 0; d < 3; ++d) red[d][threadIdx.x] += red[d][threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double o = occ[n];
    const size_t b = (size_t)blockIdx.y * gridDim.x + blockIdx.x;
    for (int d = 0; d < 3; ++d) part[3 * b + d] = o * red[d][0];
  }
}

// SelfConsistentPotential::extrapolate (SelfConsistentPotential.cc:46-73):
// v = 3 v2 - 3 v1 + 1 v0 in FP64 with the reference's operation order (no
// contraction), written as the FP64, FP32 and double-float copies the
// transforms read
__global__ void k_vextrap(const double* __restrict__ h, long long n, double* __restrict__ vr,
                          float* __restrict__ vr32, df32* __restrict__ vrdf) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double t = __dadd_rn(__dsub_rn(__dmul_rn(3.0, h[2 * n + i]), __dmul_rn(3.0, h[n + i])),
                               __dmul_rn(1.0, h[i]));
    vr[i] = t;
    const float hi = (float)t;
    vr32[i] = hi;
    vrdf[i] = df32(hi, (float)(t - (double)hi));
  }
}

qbg_status upload_occ(qbg_plan* p, const double* occ, int nst, double scale,
                             double** d_out, cudaStream_t st) {
  // the reduction buffer's tail holds per-state factors
  static_assert(sizeof(double) == 8, "");
  std::vector<double> h(std::max(nst, 1));
  for (int n = 0; n < nst; ++n) h[n] = scale * (occ ? occ[n] : 0.0);
  void** slot = &p->d_w[3];
  size_t need = sizeof(double) * h.size();
  if (*slot && p->occ_cache == h) {  // unchanged since the last upload
    *d_out = (double*)*slot;
    return QBG_OK;
  }
  QBG_TRY(ensure(slot, &p->w_bytes[3], need));
  QBG_CUDA(cudaMemcpyAsync(*slot, h.data(), need, cudaMemcpyHostToDevice, st));
  QBG_CUDA(cudaStreamSynchronize(st));  // h is a stack buffer
  p->occ_cache = h;
  *d_out = (double*)*slot;
  return QBG_OK;
}

// H psi for a block of states (FP64 in and out).  The plain form runs the
// transforms and projector GEMMs in FP64; the mixed form runs the transforms
// in FP32 and the projector GEMMs on the tensor cores.  When acc is set,
// acc += fac * (H psi) is fused into the last pass.
qbg_status hpsi_core(qbg_plan* p, const double2* psi, int ld, double2* out, int nst,
                            const double* d_occ, double* enl_part, int* enl_blocks,
                            double2* acc, int ldacc, double2 fac, cudaStream_t st) {
  const bool nl = p->nproj > 0;
  *enl_blocks = 0;
  if (p->prec == QBG_PREC_FP64) {
    if (nl) {
      if (p->fp64_gemm == QBG_GEMM_OZAKI) {
        QBG_TRY(oz_nl_apply(p, psi, ld, out, nst, d_occ, enl_part, enl_blocks, st));
      } else {
        QBG_TRY(nl_apply<double>(p, psi, ld, out, nst, d_occ, enl_part, st));
        *enl_blocks = nl_reduce_blocks(p, nst);
      }
    }
    return local_hpsi<double>(p, psi, ld, out, nst, nl, acc, ldacc, fac, st);
  }
  if (nl) {
    if (p->prec == QBG_PREC_MIXED_NL64) {
      QBG_TRY(nl_apply<double>(p, psi, ld, out, nst, d_occ, enl_part, st));
      *enl_blocks = nl_reduce_blocks(p, nst);
    } else {
      QBG_TRY(tc_nl_apply(p, psi, ld, out, nst, d_occ, enl_part, enl_blocks, st));
    }
  }
  if (p->prec == QBG_PREC_MIXED_FFT64)
    return local_hpsi<double>(p, psi, ld, out, nst, nl, acc, ldacc, fac, st);
  if (p->prec == QBG_PREC_MIXED_DF32)
    return local_hpsi<df32>(p, psi, ld, out, nst, nl, acc, ldacc, fac, st);
  return local_hpsi<float>(p, psi, ld, out, nst, nl, acc, ldacc, fac, st);
}

bool uses_tc(const qbg_plan* p) {
  return p->prec == QBG_PREC_MIXED || p->prec == QBG_PREC_MIXED_FFT64 ||
         p->prec == QBG_PREC_MIXED_DF32 ||
         (p->prec == QBG_PREC_FP64 && p->fp64_gemm == QBG_GEMM_OZAKI);
}

qbg_status check_common(qbg_plan* p, const void* a, int ld, int nst, const char* who) {
  if (!p || nst < 0 || ld < p->ngw || (nst > 0 && !a)) {
    set_error("%s: invalid argument (ld=%d, ngw=%d, nst=%d)", who, ld, p ? p->ngw : -1, nst);
    return QBG_ERR_INVALID;
  }
  return QBG_OK;
}

qbg_status ensure_nl(qbg_plan* p, cudaStream_t st) {
  if (p->nsp > 0 && !p->nl_ready) return nl_build(p, st);
  return QBG_OK;
}

// exponential(1, dt1) of ExponentialWavefunctionStepper.cc:51-148: the
// Taylor series is accumulated straight into psi (FP64); the four H
// applications ping-pong between two FP64 work buffers.
qbg_status exponential(qbg_plan* p, double2* psi, int ld, int nst, const double* d_occ,
                              double dt1, cudaStream_t st) {
  double f_re = 1.0, f_im = 0.0;
  const size_t n64 = sizeof(double2) * (size_t)ld * nst;
  QBG_TRY(ensure(&p->d_w[0], &p->w_bytes[0], n64));
  QBG_TRY(ensure(&p->d_w[1], &p->w_bytes[1], n64));
  for (int N = 1; N <= 4; ++N) {
    // factor1 *= -complex(0,1)*dt1/double(N)
    const double m_re = -0.0 * dt1 / (double)N, m_im = -1.0 * dt1 / (double)N;
    const double n_re = f_re * m_re - f_im * m_im, n_im = f_re * m_im + f_im * m_re;
    f_re = n_re;
    f_im = n_im;
    const double2 fac = make_double2(f_re, f_im);
    const double2* in = N == 1 ? psi : (const double2*)p->d_w[N & 1];
    double2* out = (double2*)p->d_w[(N - 1) & 1];
    int nb;
    QBG_TRY(hpsi_core(p, in, ld, out, nst, d_occ, nullptr, &nb, psi, ld, fac, st));
  }
  return QBG_OK;
}

}  // namespace qbg

using namespace qbg;

extern "C" {

qbg_status qbg_backward(qbg_plan* p, const double* c, int ldc, double* f, int nb, void* stream) {
  QBG_TRY(check_common(p, c, ldc, nb, "qbg_backward"));
  if (nb > 0 && !f) {
    set_error("qbg_backward: null output");
    return QBG_ERR_INVALID;
  }
  return backward<double>(p, (const double2*)c, ldc, (double2*)f, nb, (cudaStream_t)stream);
}

qbg_status qbg_forward(qbg_plan* p, double* f, double* c, int ldc, int nb, void* stream) {
  QBG_TRY(check_common(p, c, ldc, nb, "qbg_forward"));
  if (nb > 0 && !f) {
    set_error("qbg_forward: null input");
    return QBG_ERR_INVALID;
  }
  return forward<double>(p, (double2*)f, (double2*)c, ldc, nb, (cudaStream_t)stream);
}

qbg_status qbg_set_vlocal(qbg_plan* p, const double* v_r) {
  if (!p || !v_r) {
    set_error("qbg_set_vlocal: null argument");
    return QBG_ERR_INVALID;
  }
  QBG_CUDA(cudaMemcpy(p->d_vr, v_r, sizeof(double) * p->N, cudaMemcpyDefault));
  std::vector<double> h(p->N);
  QBG_CUDA(cudaMemcpy(h.data(), p->d_vr, sizeof(double) * p->N, cudaMemcpyDeviceToHost));
  std::vector<float> hf(p->N);
  std::vector<df32> hd(p->N);
  for (long long i = 0; i < p->N; ++i) {
    hf[i] = (float)h[i];
    hd[i] = df32(hf[i], (float)(h[i] - (double)hf[i]));
  }
  QBG_CUDA(cudaMemcpy(p->d_vr32, hf.data(), sizeof(float) * p->N, cudaMemcpyHostToDevice));
  QBG_CUDA(cudaMemcpy(p->d_vrdf, hd.data(), sizeof(df32) * p->N, cudaMemcpyHostToDevice));
  p->have_vr = true;
  return QBG_OK;
}

qbg_status qbg_get_vlocal(const qbg_plan* p, double* v_r) {
  if (!p || !v_r) {
    set_error("qbg_get_vlocal: null argument");
    return QBG_ERR_INVALID;
  }
  if (!p->have_vr) {
    set_error("qbg_get_vlocal: no local potential set");
    return QBG_ERR_STATE;
  }
  QBG_CUDA(cudaDeviceSynchronize());
  QBG_CUDA(cudaMemcpy(v_r, p->d_vr, sizeof(double) * p->N, cudaMemcpyDefault));
  return QBG_OK;
}

qbg_status qbg_set_nonlocal(qbg_plan* p, int nsp, const int* na, const int* lmax,
                            const double* rc, const double* wt, const double* tau) {
  if (!p || nsp < 0 || (nsp > 0 && (!na || !lmax || !rc || !wt))) {
    set_error("qbg_set_nonlocal: invalid argument");
    return QBG_ERR_INVALID;
  }
  int ntot = 0;
  for (int s = 0; s < nsp; ++s) {
    if (na[s] < 0 || lmax[s] < -1 || lmax[s] > 2) {
      set_error("qbg_set_nonlocal: species %d has na=%d lmax=%d (lmax must be -1..2)", s,
                na[s], lmax[s]);
      return QBG_ERR_INVALID;
    }
    ntot += na[s];
  }
  if (ntot > 0 && !tau) {
    set_error("qbg_set_nonlocal: null tau");
    return QBG_ERR_INVALID;
  }
  p->nsp = nsp;
  p->nl_tables = false;
  p->sp_na.assign(na, na + nsp);
  p->sp_lmax.assign(lmax, lmax + nsp);
  p->sp_rc.assign(rc, rc + nsp);
  p->sp_wt.assign(wt, wt + 3 * nsp);
  p->sp_tau.assign(tau, tau + 3 * (size_t)ntot);
  p->nl_ready = false;
  return nl_build(p, 0);
}

qbg_status qbg_set_nonlocal_tables(qbg_plan* p, int nsp, const int* na, const int* npr,
                                   const int* lproj, const double* wt, const double* twnl,
                                   const double* tau) {
  if (!p || nsp < 0 || (nsp > 0 && (!na || !npr))) {
    set_error("qbg_set_nonlocal_tables: invalid argument");
    return QBG_ERR_INVALID;
  }
  size_t rows = 0, ntot = 0;
  for (int s = 0; s < nsp; ++s) {
    if (na[s] < 0 || npr[s] < 0) {
      set_error("qbg_set_nonlocal_tables: species %d has na=%d npr=%d", s, na[s], npr[s]);
      return QBG_ERR_INVALID;
    }
    rows += npr[s];
    ntot += na[s];
  }
  if ((rows > 0 && (!lproj || !wt || !twnl)) || (ntot > 0 && !tau)) {
    set_error("qbg_set_nonlocal_tables: null table");
    return QBG_ERR_INVALID;
  }
  for (size_t r = 0; r < rows; ++r)
    if (lproj[r] < 0 || lproj[r] > 3) {
      set_error("qbg_set_nonlocal_tables: lproj[%zu] = %d (must be 0..3)", r, lproj[r]);
      return QBG_ERR_INVALID;
    }
  // kernels of any stream may still read the old tables
  QBG_CUDA(cudaDeviceSynchronize());
  const size_t bytes = sizeof(double) * rows * (size_t)p->ngw;
  if (bytes > 0) {
    QBG_TRY(ensure((void**)&p->d_twnl, &p->twnl_bytes, bytes));
    QBG_CUDA(cudaMemcpy(p->d_twnl, twnl, bytes, cudaMemcpyHostToDevice));
  }
  p->nsp = nsp;
  p->nl_tables = true;
  p->sp_na.assign(na, na + nsp);
  p->sp_npr.assign(npr, npr + nsp);
  p->sp_lproj.assign(lproj, lproj + rows);
  p->sp_wtp.assign(wt, wt + rows);
  p->sp_tau.assign(tau, tau + 3 * ntot);
  p->sp_lmax.assign(nsp, -1);
  p->sp_rc.assign(nsp, 0.0);
  p->sp_wt.assign(3 * (size_t)nsp, 0.0);
  p->nl_ready = false;
  return nl_build(p, 0);
}

qbg_status qbg_set_vector_potential(qbg_plan* p, const double* A) {
  if (!p || !A) {
    set_error("qbg_set_vector_potential: null argument");
    return QBG_ERR_INVALID;
  }
  if (A[0] == p->A[0] && A[1] == p->A[1] && A[2] == p->A[2]) return QBG_OK;
  p->A[0] = A[0];
  p->A[1] = A[1];
  p->A[2] = A[2];
  QBG_TRY(update_kinetic(p, 0));
  p->nl_ready = false;
  if (p->nsp > 0) QBG_TRY(nl_build(p, 0));
  QBG_CUDA(cudaDeviceSynchronize());
  return QBG_OK;
}

qbg_status qbg_hpsi(qbg_plan* p, const double* psi, int ld, double* hpsi, int nst,
                    const double* occ, double* enl, void* stream) {
  QBG_TRY(check_common(p, psi, ld, nst, "qbg_hpsi"));
  if (nst > 0 && !hpsi) {
    set_error("qbg_hpsi: null output");
    return QBG_ERR_INVALID;
  }
  if (nst == 0) {
    if (enl) *enl = 0.0;
    return QBG_OK;
  }
  cudaStream_t st = (cudaStream_t)stream;
  QBG_TRY(ensure_nl(p, st));
  double* d_occ = nullptr;
  QBG_TRY(upload_occ(p, occ, nst, 1.0, &d_occ, st));
  const int nbmax = p->nproj > 0 ? nl_reduce_blocks(p, nst) : 0;
  QBG_TRY(ensure((void**)&p->d_red, &p->red_bytes, sizeof(double) * std::max(nbmax, 1)));
  const double2 zero = make_double2(0.0, 0.0);
  int nb = 0;
  QBG_TRY(hpsi_core(p, (const double2*)psi, ld, (double2*)hpsi, nst, d_occ,
                    enl ? p->d_red : nullptr, &nb, nullptr, 0, zero, st));
  if (uses_tc(p)) QBG_TRY(tc_check_status(p, st));
  if (enl) {
    *enl = 0.0;
    if (nb > 0) {
      QBG_TRY(ensure_host(&p->h_red, &p->h_red_bytes, sizeof(double) * nb));
      QBG_CUDA(cudaMemcpyAsync(p->h_red, p->d_red, sizeof(double) * nb, cudaMemcpyDeviceToHost, st));
      QBG_CUDA(cudaStreamSynchronize(st));
      double s = 0.0;
      for (int i = 0; i < nb; ++i) s += p->h_red[i];
      *enl = s;
    }
  }
  return QBG_OK;
}

static qbg_status sum_device(qbg_plan* p, const double* x, long long n, double* out,
                             cudaStream_t st) {
  const int nb = 256;
  QBG_TRY(ensure((void**)&p->d_red, &p->red_bytes, sizeof(double) * nb));
  k_sum<<<nb, 256, 0, st>>>(x, n, p->d_red);
  QBG_LAUNCHED(p);
  QBG_TRY(ensure_host(&p->h_red, &p->h_red_bytes, sizeof(double) * nb));
  QBG_CUDA(cudaMemcpyAsync(p->h_red, p->d_red, sizeof(double) * nb, cudaMemcpyDeviceToHost, st));
  QBG_CUDA(cudaStreamSynchronize(st));
  double s = 0.0;
  for (int i = 0; i < nb; ++i) s += p->h_red[i];
  *out = s;
  return QBG_OK;
}

static qbg_status density_any(qbg_plan* p, const double2* psi, int ld, int nst,
                              const double* d_w, double* rho, cudaStream_t st) {
  if (p->prec == QBG_PREC_FP64 || p->prec == QBG_PREC_MIXED_FFT64)
    return density<double>(p, psi, ld, nst, d_w, rho, st);
  if (p->prec == QBG_PREC_MIXED_DF32) return density<df32>(p, psi, ld, nst, d_w, rho, st);
  return density<float>(p, psi, ld, nst, d_w, rho, st);
}

qbg_status qbg_density(qbg_plan* p, const double* psi, int ld, int nst, const double* occ,
                       double weight, double* rho, double* nel, void* stream) {
  QBG_TRY(check_common(p, psi, ld, nst, "qbg_density"));
  if (!rho) {
    set_error("qbg_density: null rho");
    return QBG_ERR_INVALID;
  }
  if (p->np1 * 16 > 16 * 256) {
    set_error("qbg_density: np1 > 256 not supported");
    return QBG_ERR_UNSUPPORTED;
  }
  cudaStream_t st = (cudaStream_t)stream;
  double* d_w = nullptr;
  QBG_TRY(upload_occ(p, occ, nst, weight / p->omega, &d_w, st));
  QBG_TRY(density_any(p, (const double2*)psi, ld, nst, d_w, rho, st));
  if (nel) {
    double s;
    QBG_TRY(sum_device(p, rho, p->N, &s, st));
    *nel = s * (p->omega / (double)p->N);
  }
  return QBG_OK;
}

qbg_status qbg_current(qbg_plan* p, const double* psi, int ld, int nst, const double* occ,
                       double nel, double* J, void* stream) {
  QBG_TRY(check_common(p, psi, ld, nst, "qbg_current"));
  if (!J) {
    set_error("qbg_current: null J");
    return QBG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  double s[3] = {0, 0, 0};
  if (nst > 0 && p->ngw > 0) {
    double* d_occ = nullptr;
    QBG_TRY(upload_occ(p, occ, nst, 1.0, &d_occ, st));
    const int gx = std::min(64, (p->ngw + 255) / 256);
    const size_t nb = (size_t)gx * nst;
    QBG_TRY(ensure((void**)&p->d_red, &p->red_bytes, sizeof(double) * 3 * nb));
    k_current<<<dim3(gx, nst), 256, 0, st>>>((const double2*)psi, ld, p->ngw, p->d_kpgx, d_occ,
                                            p->d_red);
    QBG_LAUNCHED(p);
    QBG_TRY(ensure_host(&p->h_red, &p->h_red_bytes, sizeof(double) * 3 * nb));
    QBG_CUDA(cudaMemcpyAsync(p->h_red, p->d_red, sizeof(double) * 3 * nb,
                             cudaMemcpyDeviceToHost, st));
    QBG_CUDA(cudaStreamSynchronize(st));
    for (size_t b = 0; b < nb; ++b)
      for (int d = 0; d < 3; ++d) s[d] += p->h_red[3 * b + d];
  }
  for (int d = 0; d < 3; ++d) J[d] = -s[d] + p->A[d] * nel;
  return QBG_OK;
}

// SlaterDet::gram (SlaterDet.cc:1043-1143), complex branch, norm-conserving:
// S = C^H C (herk), S = L L^H (potrf, lower), C <- C L^{-H} (trsm).  The two
// nst^2 ngw products run on the device in FP64; the nst^3 Cholesky factor
// and the triangular inverse are formed on the host (a 432-state overlap is
// 3 MB) in FP64, in the column order of the LAPACK algorithms.
qbg_status qbg_gram(qbg_plan* p, double* psi_, int ld, int nst, void* stream) {
  QBG_TRY(check_common(p, psi_, ld, nst, "qbg_gram"));
  if (nst == 0) return QBG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  double2* psi = (double2*)psi_;
  const size_t nn = (size_t)nst * nst;
  QBG_TRY(ensure(&p->d_w[2], &p->w_bytes[2], sizeof(double2) * std::max(nn, (size_t)ld * nst)));
  double2* S = (double2*)p->d_w[2];
  QBG_TRY(gram_overlap(p, psi, ld, nst, S, st));
  std::vector<std::complex<double>> h(nn);
  QBG_CUDA(cudaMemcpyAsync(h.data(), S, sizeof(double2) * nn, cudaMemcpyDeviceToHost, st));
  QBG_CUDA(cudaStreamSynchronize(st));
  // A(i, j) = <psi_i|psi_j> = h[j*nst + i]; lower Cholesky A = L L^H in place
  auto A = [&](int i, int j) -> std::complex<double>& { return h[(size_t)j * nst + i]; };
  for (int j = 0; j < nst; ++j) {
    double d = A(j, j).real();
    for (int k = 0; k < j; ++k) d -= std::norm(A(j, k));
    if (!(d > 0.0)) {
      set_error("qbg_gram: the overlap matrix is not positive definite at state %d "
                "(linearly dependent states)", j);
      return QBG_ERR_DIVERGED;
    }
    const double ljj = std::sqrt(d);
    A(j, j) = ljj;
    for (int i = j + 1; i < nst; ++i) {
      std::complex<double> t = A(i, j);
      for (int k = 0; k < j; ++k) t -= A(i, k) * std::conj(A(j, k));
      A(i, j) = t / ljj;
    }
  }
  // U = L^{-H} (upper triangular); psi'_n = sum_m psi_m U(m, n); the device
  // product wants T[n][m] = U(m, n)
  std::vector<std::complex<double>> Li(nn, 0.0);  // L^{-1}, lower
  for (int j = 0; j < nst; ++j) {
    Li[(size_t)j * nst + j] = 1.0 / A(j, j);
    for (int i = j + 1; i < nst; ++i) {
      std::complex<double> t = 0.0;
      for (int k = j; k < i; ++k) t -= A(i, k) * Li[(size_t)j * nst + k];
      Li[(size_t)j * nst + i] = t / A(i, i);
    }
  }
  std::vector<double2> T(nn, make_double2(0.0, 0.0));
  for (int n = 0; n < nst; ++n)
    for (int m = 0; m <= n; ++m) {
      // U(m, n) = conj(Linv(n, m))
      const std::complex<double> u = std::conj(Li[(size_t)m * nst + n]);
      T[(size_t)n * nst + m] = make_double2(u.real(), u.imag());
    }
  QBG_TRY(ensure(&p->d_w[3], &p->w_bytes[3], sizeof(double2) * nn));
  double2* dT = (double2*)p->d_w[3];
  p->occ_cache.clear();  // d_w[3] held the per-state factors
  QBG_CUDA(cudaMemcpyAsync(dT, T.data(), sizeof(double2) * nn, cudaMemcpyHostToDevice, st));
  double2* out = (double2*)p->d_w[2];
  QBG_TRY(gram_apply(p, psi, ld, nst, dT, out, ld, st));
  QBG_CUDA(cudaMemcpy2DAsync(psi, sizeof(double2) * ld, out, sizeof(double2) * ld,
                             sizeof(double2) * p->ngw, nst, cudaMemcpyDeviceToDevice, st));
  QBG_CUDA(cudaStreamSynchronize(st));  // T is a host stack buffer
  return QBG_OK;
}

qbg_status qbg_set_aetrs(qbg_plan* p, int on) {
  if (!p) {
    set_error("qbg_set_aetrs: null plan");
    return QBG_ERR_INVALID;
  }
  p->aetrs = on != 0;
  p->aetrs_stored = 0;
  return QBG_OK;
}

qbg_status qbg_etrs_step(qbg_plan* p, double* psi_, int ld, int nst, const double* occ,
                         double dt, const double* A_t, const double* A_tdt, double* rho_mid,
                         double* nel, void* stream) {
  QBG_TRY(check_common(p, psi_, ld, nst, "qbg_etrs_step"));
  if (nst == 0) return QBG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  double2* psi = (double2*)psi_;
  if (A_t) QBG_TRY(qbg_set_vector_potential(p, A_t));
  QBG_TRY(ensure_nl(p, st));
  double* d_occ = nullptr;
  QBG_TRY(upload_occ(p, occ, nst, 1.0 / p->omega, &d_occ, st));
  const double dt1 = 0.5 * dt;
  double* rho = rho_mid;
  if (!rho || p->selfconsistent) {
    QBG_TRY(ensure((void**)&p->d_rho, &p->rho_bytes, sizeof(double) * (size_t)p->N));
    if (!rho) rho = p->d_rho;
  }
  if (p->selfconsistent) {
    // loop top: H(t) from the density of psi(t) (EhrenSampleStepper.cc:322-329)
    QBG_TRY(density_any(p, psi, ld, nst, d_occ, p->d_rho, st));
    QBG_TRY(vhxc_update(p, p->d_rho, st));
  }
  if (p->aetrs) {
    // AETRS preupdate (ExponentialWavefunctionStepper.cc:158-163): keep the
    // potential of H(t); from the third stored step on, the second half step
    // runs with the potential extrapolated from the last three
    // (:201-227), and update() does nothing (:247)
    const size_t nb = sizeof(double) * (size_t)p->N;
    QBG_TRY(ensure((void**)&p->d_vhist, &p->vhist_bytes, 3 * nb));
    QBG_CUDA(cudaMemcpyAsync(p->d_vhist, p->d_vhist + p->N, nb, cudaMemcpyDeviceToDevice, st));
    QBG_CUDA(cudaMemcpyAsync(p->d_vhist + p->N, p->d_vhist + 2 * p->N, nb,
                             cudaMemcpyDeviceToDevice, st));
    QBG_CUDA(cudaMemcpyAsync(p->d_vhist + 2 * p->N, p->d_vr, nb, cudaMemcpyDeviceToDevice, st));
    if (p->aetrs_stored < 3) p->aetrs_stored++;
    if (p->aetrs_stored >= 3) {
      QBG_TRY(exponential(p, psi, ld, nst, d_occ, dt1, st));
      k_vextrap<<<2 * 152 * 4, 256, 0, st>>>(p->d_vhist, p->N, p->d_vr, p->d_vr32, p->d_vrdf);
      QBG_LAUNCHED(p);
      QBG_TRY(exponential(p, psi, ld, nst, d_occ, dt1, st));
      if (rho_mid || nel) {
        // no predicted state exists in this step: the density returned is
        // that of psi(t+dt)
        QBG_TRY(density_any(p, psi, ld, nst, d_occ, rho, st));
        if (nel) {
          double s;
          QBG_TRY(sum_device(p, rho, p->N, &s, st));
          *nel = s * (p->omega / (double)p->N);
        }
      }
      if (A_tdt) QBG_TRY(qbg_set_vector_potential(p, A_tdt));
      if (uses_tc(p) && p->check_every_step) QBG_TRY(tc_check_status(p, st));
      return QBG_OK;
    }
  }
  // preupdate: psi(t) -> psi(t+dt/2) (kept), -> predicted psi(t+dt) in X
  QBG_TRY(exponential(p, psi, ld, nst, d_occ, dt1, st));
  const size_t n64 = sizeof(double2) * (size_t)ld * nst;
  QBG_TRY(ensure(&p->d_w[2], &p->w_bytes[2], n64));
  double2* X = (double2*)p->d_w[2];
  {
    dim3 g((p->ngw + 255) / 256, nst);
    k_copy_cols<<<g, 256, 0, st>>>(psi, ld, X, ld, p->ngw);
    QBG_LAUNCHED(p);
  }
  QBG_TRY(exponential(p, X, ld, nst, d_occ, dt1, st));
  // update: density of the predicted state (hamil_cd()->update_density),
  // then H(t+dt) and the last half step from psi(t+dt/2)
  QBG_TRY(density_any(p, X, ld, nst, d_occ, rho, st));
  if (p->selfconsistent) QBG_TRY(vhxc_update(p, rho, st));
  if (nel) {
    double s;
    QBG_TRY(sum_device(p, rho, p->N, &s, st));
    *nel = s * (p->omega / (double)p->N);
  }
  if (A_tdt) QBG_TRY(qbg_set_vector_potential(p, A_tdt));
  QBG_TRY(exponential(p, psi, ld, nst, d_occ, dt1, st));
  if (uses_tc(p) && p->check_every_step) QBG_TRY(tc_check_status(p, st));
  return QBG_OK;
}

}  // extern "C"
