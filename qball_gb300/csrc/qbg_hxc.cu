// qbg_hxc.cu -- Hartree + LDA exchange-correlation potential from the charge
// density: EnergyFunctional::update_hamiltonian + update_vhxc
// (EnergyFunctional.cc:300-520, TD branch), XCPotential::update
// (XCPotential.cc:130-190) and LDAFunctional::xc_unpolarized
// (functionals/LDAFunctional.cc:102-160).
//
// The density basis lives in a second plan (vplan) on the same grid, built
// in FP64 whatever the main plan's precision: one density transform, one
// potential transform and two grid sweeps per update, against the hundreds
// of wavefunction transforms of an ETRS step.
//   k_rho_pack  f = Omega rho + 0i                          (N complex)
//   forward_v   rho_G = f(G) on the density sphere
//   k_hartree   v_G = vion_G + 4 pi (rho_G/Omega + rhopst_G) g2i, with the
//               E_H and E_ps partial sums
//   backward_v  f = v(r)
//   k_lda       v_r = vxc(rho) + Re f, written as FP64, FP32 and
//               double-float copies, with the E_xc partial sums
// Energies stay as per-block partials on the device until a caller asks.
#include <algorithm>
#include <cmath>
#include <vector>

#include "qbg_internal.h"

namespace qbg {

#define QBG_TRY(x)                \
  do {                            \
    qbg_status s_ = (x);          \
    if (s_ != QBG_OK) return s_;  \
  } while (0)

constexpr int kHxcBlocks = 256;
constexpr int kHxcThreads = 256;

// Exchange of the uniform electron gas plus the Perdew-Zunger (1981) fit of
// the Ceperley-Alder correlation energy, spin unpolarised, Hartree units.
// With rs = (3/(4 pi rho))^(1/3): e_x = (3/4) v_x, v_x = c3 / rs;
// e_c = A ln rs + B + C rs ln rs + D rs (rs < 1) or
// gamma / (1 + beta1 sqrt(rs) + beta2 rs) (rs >= 1); v_c = e_c - (rs/3)
// de_c/drs.  C and D make e_c and v_c continuous at rs = 1.
__device__ __forceinline__ void lda_pz(double rh, double& e, double& v) {
  const double c1 = 0.6203504908994001;  // (3/(4 pi))^(1/3)
  const double c3 = -0.610887057711;     // -(9 pi / 4)^(1/3) / pi
  const double A = 0.0311, B = -0.048, b1 = 1.0529, b2 = 0.3334, G = -0.1423;
  const double D = G / (1.0 + b1 + b2) - B;
  const double C = -A - D - G * ((b1 / 2.0 + b2) / ((1.0 + b1 + b2) * (1.0 + b1 + b2)));
  e = 0.0;
  v = 0.0;
  if (rh > 0.0) {
    const double rs = c1 / cbrt(rh);
    const double vx = c3 / rs, ex = 0.75 * vx;
    double ec, vc;
    if (rs < 1.0) {
      const double lr = log(rs);
      ec = A * lr + B + C * rs * lr + D * rs;
      vc = A * lr + (B - A / 3.0) + (2.0 / 3.0) * C * rs * lr + ((2.0 * D - C) / 3.0) * rs;
    } else {
      const double sr = sqrt(rs);
      const double den = 1.0 + b1 * sr + b2 * rs;
      ec = G / den;
      vc = ec * (1.0 + (7.0 / 6.0) * b1 * sr + (4.0 / 3.0) * b2 * rs) / den;
    }
    e = ex + ec;
    v = vx + vc;
  }
}

__device__ __forceinline__ double block_sum(double x, double* red) {
  red[threadIdx.x] = x;
  __syncthreads();
  for (int k = kHxcThreads / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kHxcThreads)
k_rho_pack(const double* __restrict__ rho, long long n, double omega, double2* __restrict__ f) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    f[i] = make_double2(omega * rho[i], 0.0);
}

// part[0][b]: sum (rho_G + rhopst)^2 g2i; part[1][b]: sum Re(conj(rho_G) vion)
__global__ void __launch_bounds__(kHxcThreads)
k_hartree(double2* __restrict__ vg, int ngv, const double* __restrict__ g2i,
          const double2* __restrict__ vion, const double2* __restrict__ rhopst,
          double omega_inv, double* __restrict__ part) {
  __shared__ double red[kHxcThreads];
  const double fpi = 4.0 * M_PI;
  double eh = 0.0, ep = 0.0;
  for (int ig = blockIdx.x * blockDim.x + threadIdx.x; ig < ngv; ig += gridDim.x * blockDim.x) {
    const double2 r = vg[ig];
    const double re = omega_inv * r.x, im = omega_inv * r.y;
    const double2 vi = vion[ig];
    ep += re * vi.x + im * vi.y;
    double tr = re, ti = im;
    if (rhopst) {
      tr += rhopst[ig].x;
      ti += rhopst[ig].y;
    }
    const double gi = g2i[ig];
    eh += (tr * tr + ti * ti) * gi;
    vg[ig] = make_double2(vi.x + fpi * tr * gi, vi.y + fpi * ti * gi);
  }
  eh = block_sum(eh, red);
  ep = block_sum(ep, red);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = eh;
    part[kHxcBlocks + blockIdx.x] = ep;
  }
}

// part[2][b]: sum rho e_xc(rho)
__global__ void __launch_bounds__(kHxcThreads)
k_lda(const double2* __restrict__ f, const double* __restrict__ rho, long long n,
      double* __restrict__ vr, float* __restrict__ vr32, df32* __restrict__ vrdf,
      double* __restrict__ part) {
  __shared__ double red[kHxcThreads];
  double ex = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double r = rho[i];
    double e, v;
    lda_pz(r, e, v);
    ex += r * e;
    const double t = v + f[i].x;
    vr[i] = t;
    const float hi = (float)t;
    vr32[i] = hi;
    vrdf[i] = df32(hi, (float)(t - (double)hi));
  }
  ex = block_sum(ex, red);
  if (threadIdx.x == 0) part[2 * kHxcBlocks + blockIdx.x] = ex;
}

void hxc_release(qbg_plan* p) {
  if (p->vplan) {
    qbg_plan_destroy(p->vplan);
    p->vplan = nullptr;
  }
  void* bufs[] = {p->d_g2i, p->d_vion, p->d_rhopst, p->d_vg, p->d_vf, p->d_hxc_red};
  for (void* b : bufs)
    if (b) cudaFree(b);
  p->d_g2i = nullptr;
  p->d_vion = nullptr;
  p->d_rhopst = nullptr;
  p->d_vg = nullptr;
  p->d_vf = nullptr;
  p->d_hxc_red = nullptr;
  p->have_ionic = false;
  p->selfconsistent = false;
}

static qbg_status density_to_g(qbg_plan* p, const double* rho, double2* rhog, cudaStream_t st) {
  k_rho_pack<<<kHxcBlocks, kHxcThreads, 0, st>>>(rho, p->N, p->omega, p->d_vf);
  QBG_LAUNCHED(p);
  return forward<double>(p->vplan, p->d_vf, rhog, p->vplan->ngw, 1, st);
}

qbg_status vhxc_update(qbg_plan* p, const double* rho, cudaStream_t st) {
  qbg_plan* vp = p->vplan;
  QBG_TRY(density_to_g(p, rho, p->d_vg, st));
  k_hartree<<<kHxcBlocks, kHxcThreads, 0, st>>>(p->d_vg, vp->ngw, p->d_g2i, p->d_vion,
                                                p->d_rhopst, 1.0 / p->omega, p->d_hxc_red);
  QBG_LAUNCHED(p);
  QBG_TRY(backward<double>(vp, p->d_vg, vp->ngw, p->d_vf, 1, st));
  k_lda<<<kHxcBlocks, kHxcThreads, 0, st>>>(p->d_vf, rho, p->N, p->d_vr, p->d_vr32, p->d_vrdf,
                                            p->d_hxc_red);
  QBG_LAUNCHED(p);
  p->have_vr = true;
  return QBG_OK;
}

static qbg_status check_hxc(qbg_plan* p, const char* who) {
  if (!p) {
    set_error("%s: null plan", who);
    return QBG_ERR_INVALID;
  }
  if (!p->vplan) {
    set_error("%s: no density basis (qbg_set_density_basis)", who);
    return QBG_ERR_STATE;
  }
  return QBG_OK;
}

}  // namespace qbg

using namespace qbg;

extern "C" {

qbg_status qbg_set_density_basis(qbg_plan* p, const qbg_basis_desc* vb) {
  if (!p || !vb || vb->ngw <= 0) {
    set_error("qbg_set_density_basis: invalid argument");
    return QBG_ERR_INVALID;
  }
  hxc_release(p);
  qbg_plan* vp = nullptr;
  qbg_status s = qbg_plan_create(vb, p->np0, p->np1, p->np2, QBG_PREC_FP64, &vp);
  if (s != QBG_OK) return s;  // the error text names the misfit
  p->vplan = vp;
  vp->chunk = 1;
  const int ngv = vb->ngw;
  // g2i = (1/|G|)^2, 0 at G = 0 (Basis::update_g, Basis.cc:730-739)
  std::vector<double> g2i(ngv);
  for (int i = 0; i < ngv; ++i) {
    const double x = vb->kpgx[i], y = vb->kpgx[ngv + i], z = vb->kpgx[2 * (size_t)ngv + i];
    const double g = std::sqrt(x * x + y * y + z * z);
    const double gi = g > 0.0 ? 1.0 / g : 0.0;
    g2i[i] = gi * gi;
  }
  auto fail = [p](qbg_status st) {
    hxc_release(p);
    return st;
  };
  cudaError_t e = cudaMalloc(&p->d_g2i, sizeof(double) * ngv);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_vion, sizeof(double2) * ngv);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_vg, sizeof(double2) * ngv);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_vf, sizeof(double2) * (size_t)p->N);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_hxc_red, sizeof(double) * 3 * kHxcBlocks);
  if (e == cudaSuccess)
    e = cudaMemcpy(p->d_g2i, g2i.data(), sizeof(double) * ngv, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(p->d_vion, 0, sizeof(double2) * ngv);
  if (e == cudaSuccess) e = cudaMemset(p->d_hxc_red, 0, sizeof(double) * 3 * kHxcBlocks);
  if (e != cudaSuccess) return fail(cuda_status(e, "qbg_set_density_basis"));
  return QBG_OK;
}

qbg_status qbg_set_ionic_terms(qbg_plan* p, const double* vion_g, const double* rhopst_g) {
  QBG_TRY(check_hxc(p, "qbg_set_ionic_terms"));
  if (!vion_g) {
    set_error("qbg_set_ionic_terms: null vion_g");
    return QBG_ERR_INVALID;
  }
  const size_t bytes = sizeof(double2) * p->vplan->ngw;
  QBG_CUDA(cudaMemcpy(p->d_vion, vion_g, bytes, cudaMemcpyHostToDevice));
  if (rhopst_g) {
    if (!p->d_rhopst) QBG_CUDA(cudaMalloc(&p->d_rhopst, bytes));
    QBG_CUDA(cudaMemcpy(p->d_rhopst, rhopst_g, bytes, cudaMemcpyHostToDevice));
  } else if (p->d_rhopst) {
    QBG_CUDA(cudaFree(p->d_rhopst));
    p->d_rhopst = nullptr;
  }
  p->have_ionic = true;
  return QBG_OK;
}

qbg_status qbg_density_g(qbg_plan* p, const double* rho, double* rhog, void* stream) {
  QBG_TRY(check_hxc(p, "qbg_density_g"));
  if (!rho || !rhog) {
    set_error("qbg_density_g: null argument");
    return QBG_ERR_INVALID;
  }
  return density_to_g(p, rho, (double2*)rhog, (cudaStream_t)stream);
}

qbg_status qbg_update_vhxc(qbg_plan* p, const double* rho, double* en, void* stream) {
  QBG_TRY(check_hxc(p, "qbg_update_vhxc"));
  if (!rho) {
    set_error("qbg_update_vhxc: null rho");
    return QBG_ERR_INVALID;
  }
  if (!p->have_ionic) {
    set_error("qbg_update_vhxc: no ionic terms (qbg_set_ionic_terms)");
    return QBG_ERR_STATE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  QBG_TRY(vhxc_update(p, rho, st));
  if (en) {
    std::vector<double> h(3 * kHxcBlocks);
    QBG_CUDA(cudaMemcpyAsync(h.data(), p->d_hxc_red, sizeof(double) * h.size(),
                             cudaMemcpyDeviceToHost, st));
    QBG_CUDA(cudaStreamSynchronize(st));
    double s[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < 3; ++k)
      for (int b = 0; b < kHxcBlocks; ++b) s[k] += h[k * kHxcBlocks + b];
    // complex basis: vfact = 0.5 (EnergyFunctional.cc:494-497)
    en[0] = 0.5 * p->omega * (4.0 * M_PI) * s[0];
    en[1] = s[2] * p->omega / (double)p->N;  // XCPotential.cc:186
    en[2] = s[1] * p->omega;                 // EnergyFunctional.cc:461-465
  }
  return QBG_OK;
}

qbg_status qbg_set_selfconsistent(qbg_plan* p, int on) {
  if (!p) {
    set_error("qbg_set_selfconsistent: null plan");
    return QBG_ERR_INVALID;
  }
  if (on && (!p->vplan || !p->have_ionic)) {
    set_error("qbg_set_selfconsistent: needs qbg_set_density_basis and qbg_set_ionic_terms");
    return QBG_ERR_STATE;
  }
  p->selfconsistent = on != 0;
  return QBG_OK;
}

}  // extern "C"
