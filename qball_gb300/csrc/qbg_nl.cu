// qbg_nl.cu -- Kleinman-Bylander nonlocal projectors.
//
// NonLocalPotential::energy (NonLocalPotential.cc:1908-2170) recomputes the
// structure factors and the projector block anl = twnl (-i)^l exp(-i(k+G-A).tau)
// on every call.  Atoms are frozen on this path and A changes only when the
// caller sets a new vector potential, so the table anl[p][g] is built once
// per A (nl_build) and kept resident in HBM; every H application then runs
//   GEMM1  fnl[n][p] = sum_g conj(anl[p][g]) psi[n][g]      (split-K, FP64
//                                                            partial sums)
//   scale  fnl *= D_p/Omega, E_nl += occ_n D_p/Omega |fnl|^2
//   GEMM2  out[n][g] = sum_p anl[p][g] fnl[n][p]
// GEMM2 writes the nonlocal part as the first term of H psi, i.e. it also
// performs the "dwf.clear()" of EnergyFunctional::energy.
#include <algorithm>
#include <vector>

#include "qbg_internal.h"

namespace qbg {

// projector descriptor: l, m index within l, species radius, weight/omega;
// row >= 0: the radial-angular factor is row `row` of the caller's tables
// (qbg_set_nonlocal_tables), else the synthetic radial form
struct ProjDesc {
  int l, m;
  double rc, wt;
  double tau[3];
  int row;
};

// One atom's projectors: p = p0 + ipr * stride for ipr < npr (the index
// ia + ipr*nblk of NonLocalPotential.cc:2000 inside the atom's block).
struct AtomDesc {
  int p0, stride, npr, pad;
  double rc;
  double tau[3];
};

// update_twnl (NonLocalPotential.cc:306-760) for the synthetic radial form,
// evaluated at k+G-A, times (-i)^l exp(-i (k+G-A).tau)  (:1962-2037).  One
// thread per (G, atom): the structure phase, |k+G-A| and the radial
// Gaussian are computed once and shared by the atom's projectors (FP64
// transcendentals are the cost of this kernel on GB300).  With caller
// tables (pd[p].row >= 0) the factor twnl[row][g] is taken as given, for
// l = 0..3.
__global__ void k_anl(const double* __restrict__ kpgx, const double* __restrict__ kpg2A,
                      int ngw, double A0, double A1, double A2,
                      const AtomDesc* __restrict__ ad, const ProjDesc* __restrict__ pd,
                      const double* __restrict__ twnl, double2* __restrict__ anl) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ngw) return;
  const AtomDesc at = ad[blockIdx.y];
  const double kx = kpgx[g] - A0, ky = kpgx[ngw + g] - A1, kz = kpgx[2 * ngw + g] - A2;
  const double k2 = kpg2A[g];
  const double tg = sqrt(k2);
  const double tgi = k2 > 0.0 ? 1.0 / sqrt(k2) : 0.0;
  const double e = exp(-0.5 * tg * tg * at.rc * at.rc);
  const double pi = 3.14159265358979323846, fpi = 4.0 * pi;
  // kpgr = -(k+G-A).tau, rounded term by term as the reference's dgemm
  double kpgr = __dmul_rn(-at.tau[0], kx);
  kpgr = __dadd_rn(kpgr, __dmul_rn(-at.tau[1], ky));
  kpgr = __dadd_rn(kpgr, __dmul_rn(-at.tau[2], kz));
  double s, c;
  sincos(kpgr, &s, &c);
  for (int ipr = 0; ipr < at.npr; ++ipr) {
    const int p = at.p0 + ipr * at.stride;
    const ProjDesc d = pd[p];
    double t;
    if (d.row >= 0) {
      t = twnl[(size_t)d.row * ngw + g];
    } else if (d.l == 0) {
      t = sqrt(1.0 / fpi) * e;
    } else if (d.l == 1) {
      const double s34pi = sqrt(3.0 / fpi);
      const double cm = d.m == 0 ? kx : (d.m == 1 ? ky : kz);
      t = (s34pi * cm * tgi) * (tg * e);
    } else {
      const double s54pi = sqrt(5.0 / fpi), s3 = sqrt(3.0);
      const double tgi2 = tgi * tgi;
      double y;
      switch (d.m) {
        case 0: y = s54pi * 0.5 * (3.0 * (kz * kz * tgi2) - 1.0); break;
        case 1: y = s54pi * 0.5 * s3 * (kx * kx * tgi2 - ky * ky * tgi2); break;
        case 2: y = s54pi * s3 * (kx * ky * tgi2); break;
        case 3: y = s54pi * s3 * (ky * kz * tgi2); break;
        default: y = s54pi * s3 * (kx * kz * tgi2); break;
      }
      t = y * (tg * tg * e);
    }
    double re, im;
    if (d.l == 0) {
      re = t * c;
      im = t * s;
    } else if (d.l == 1) {
      re = t * s;
      im = -t * c;
    } else if (d.l == 2) {
      re = -t * c;
      im = -t * s;
    } else {
      re = -t * s;
      im = t * c;
    }
    anl[(size_t)p * ngw + g] = make_double2(re, im);
  }
}

__global__ void k_kpg2A(const double* __restrict__ kpgx, int ngw, double A0, double A1,
                        double A2, double* __restrict__ kpg2A, float* __restrict__ kpg2A32) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ngw) return;
  const double kx = kpgx[g], ky = kpgx[ngw + g], kz = kpgx[2 * ngw + g];
  // VectorPotential::get_kpgpa2 (VectorPotential.h:84-95)
  double k2 = __dadd_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)), __dmul_rn(kz, kz));
  const double value2 = __dadd_rn(__dadd_rn(__dmul_rn(A0, A0), __dmul_rn(A1, A1)), __dmul_rn(A2, A2));
  double t = __dadd_rn(k2, value2);
  t = __dsub_rn(t, __dmul_rn(__dmul_rn(2.0, A0), kx));
  t = __dsub_rn(t, __dmul_rn(__dmul_rn(2.0, A1), ky));
  t = __dsub_rn(t, __dmul_rn(__dmul_rn(2.0, A2), kz));
  kpg2A[g] = t;
  kpg2A32[g] = (float)t;
}

qbg_status update_kinetic(qbg_plan* p, cudaStream_t st) {
  if (p->ngw == 0) return QBG_OK;
  k_kpg2A<<<(p->ngw + 255) / 256, 256, 0, st>>>(p->d_kpgx, p->ngw, p->A[0], p->A[1], p->A[2],
                                                p->d_kpg2A, p->d_kpg2A32);
  QBG_LAUNCHED(p);
  return QBG_OK;
}

// projector order: species, atom blocks of <= 128 atoms, projector ipr
// (l, then m), atom within the block -- the index ia + ipr*nblk of
// NonLocalPotential.cc:2000 taken block by block.
static void proj_descs(const qbg_plan* p, std::vector<ProjDesc>& pd, std::vector<double>& wt,
                       std::vector<AtomDesc>& ad) {
  int namax = 0;
  for (int s = 0; s < p->nsp; ++s) namax = std::max(namax, p->sp_na[s]);
  const int nbs = std::max(1, std::min(namax, 128));
  int atom0 = 0;
  if (p->nl_tables) {
    // caller tables: npr[s] projectors of species s with l = lproj, weight wt
    int row0 = 0;
    for (int s = 0; s < p->nsp; ++s) {
      const int na = p->sp_na[s], npr = p->sp_npr[s];
      for (int b0 = 0; b0 < na; b0 += nbs) {
        const int b1 = std::min(na, b0 + nbs);
        for (int ia = b0; ia < b1; ++ia) {
          AtomDesc a;
          a.p0 = (int)pd.size() + (ia - b0);
          a.stride = b1 - b0;
          a.npr = npr;
          a.pad = 0;
          a.rc = 0.0;
          for (int j = 0; j < 3; ++j) a.tau[j] = p->sp_tau[3 * (size_t)(atom0 + ia) + j];
          if (npr > 0) ad.push_back(a);
        }
        for (int ipr = 0; ipr < npr; ++ipr)
          for (int ia = b0; ia < b1; ++ia) {
            ProjDesc d;
            d.l = p->sp_lproj[row0 + ipr];
            d.m = 0;
            d.rc = 0.0;
            d.wt = p->sp_wtp[row0 + ipr] / p->omega;
            for (int j = 0; j < 3; ++j) d.tau[j] = p->sp_tau[3 * (size_t)(atom0 + ia) + j];
            d.row = row0 + ipr;
            pd.push_back(d);
            wt.push_back(d.wt);
          }
      }
      atom0 += na;
      row0 += npr;
    }
    return;
  }
  for (int s = 0; s < p->nsp; ++s) {
    const int na = p->sp_na[s], lmax = p->sp_lmax[s];
    for (int b0 = 0; b0 < na; b0 += nbs) {
      const int b1 = std::min(na, b0 + nbs);
      for (int ia = b0; ia < b1; ++ia) {
        AtomDesc a;
        a.p0 = (int)pd.size() + (ia - b0);
        a.stride = b1 - b0;
        a.npr = (lmax + 1) * (lmax + 1);
        a.pad = 0;
        a.rc = p->sp_rc[s];
        for (int j = 0; j < 3; ++j) a.tau[j] = p->sp_tau[3 * (size_t)(atom0 + ia) + j];
        if (a.npr > 0) ad.push_back(a);
      }
      for (int l = 0; l <= lmax; ++l)
        for (int m = 0; m < 2 * l + 1; ++m)
          for (int ia = b0; ia < b1; ++ia) {
            ProjDesc d;
            d.l = l;
            d.m = m;
            d.rc = p->sp_rc[s];
            d.wt = p->sp_wt[3 * s + l] / p->omega;
            for (int j = 0; j < 3; ++j) d.tau[j] = p->sp_tau[3 * (size_t)(atom0 + ia) + j];
            d.row = -1;
            pd.push_back(d);
            wt.push_back(d.wt);
          }
    }
    atom0 += na;
  }
}

// Builds the projector table for the plan's A.  When only A (or the atom
// positions) changed, the table and its tensor-core pieces are rebuilt in
// their existing buffers: no allocation, no device-wide synchronisation
// from cudaFree on the per-step path of a laser-driven run.
qbg_status nl_build(qbg_plan* p, cudaStream_t st) {
  std::vector<ProjDesc> pd;
  std::vector<double> wt;
  std::vector<AtomDesc> ad;
  proj_descs(p, pd, wt, ad);
  const int P = (int)pd.size();
  const size_t n = (size_t)P * p->ngw;
  const bool same = P == p->nproj && p->d_anl && p->anl_elems == n && n > 0;
  if (same) {
    // kernels of any stream may still read the old table
    QBG_CUDA(cudaDeviceSynchronize());
    tc_invalidate(p);
    oz_invalidate(p);
  } else {
    tc_release(p);
    oz_release(p);
    void* bufs[] = {p->d_ptau, p->d_pwt, p->d_anl, p->d_anl32, p->d_pdesc, p->d_adesc};
    for (void* b : bufs)
      if (b) cudaFree(b);
    p->d_ptau = nullptr;
    p->d_pwt = nullptr;
    p->d_anl = nullptr;
    p->d_anl32 = nullptr;
    p->d_pdesc = nullptr;
    p->d_adesc = nullptr;
    p->anl_elems = 0;
  }
  p->nl_natoms = (int)ad.size();
  p->nproj = P;
  p->nl_ready = true;
  p->nl_version++;
  if (P == 0 || p->ngw == 0) return QBG_OK;
  if (!same) {
    QBG_CUDA(cudaMalloc(&p->d_pdesc, sizeof(ProjDesc) * P));
    QBG_CUDA(cudaMalloc(&p->d_adesc, sizeof(AtomDesc) * ad.size()));
    QBG_CUDA(cudaMalloc(&p->d_pwt, sizeof(double) * P));
    QBG_CUDA(cudaMalloc(&p->d_anl, sizeof(double2) * n));
    p->anl_elems = n;
  }
  // pageable host sources: these copies complete before returning
  QBG_CUDA(cudaMemcpy(p->d_pdesc, pd.data(), sizeof(ProjDesc) * P, cudaMemcpyHostToDevice));
  QBG_CUDA(cudaMemcpy(p->d_pwt, wt.data(), sizeof(double) * P, cudaMemcpyHostToDevice));
  QBG_CUDA(cudaMemcpy(p->d_adesc, ad.data(), sizeof(AtomDesc) * ad.size(),
                      cudaMemcpyHostToDevice));
  dim3 grid((p->ngw + 255) / 256, (unsigned)ad.size());
  k_anl<<<grid, 256, 0, st>>>(p->d_kpgx, p->d_kpg2A, p->ngw, p->A[0], p->A[1], p->A[2],
                              (const AtomDesc*)p->d_adesc, (const ProjDesc*)p->d_pdesc,
                              p->d_twnl, p->d_anl);
  p->launches++;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_status(e, "k_anl");
  return QBG_OK;
}

// ------------------------------------------------------------------ GEMMs
constexpr int GT = 64;   // output tile edge
constexpr int GK = 16;   // k step

// part[z][n][p] = sum_{g in split z} conj(anl[p][g]) psi[n][g], g < ngw;
// anl rows lda apart
template <typename T>
__global__ void __launch_bounds__(256)
k_fnl(const cplx<T>* __restrict__ anl, int lda, int ngw, int nproj,
      const cplx<T>* __restrict__ psi, int ld, int nst, double2* __restrict__ part, int kchunk) {
  using C = cplx<T>;
  __shared__ C As[GK][GT];
  __shared__ C Bs[GK][GT];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int p0 = blockIdx.x * GT, n0 = blockIdx.y * GT;
  const int kb = blockIdx.z * kchunk, ke = min(ngw, kb + kchunk);
  T ar[4][4], ai[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) ar[i][j] = ai[i][j] = T(0);
  for (int k0 = kb; k0 < ke; k0 += GK) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = tid + 256 * q, r = e >> 4, kk = e & 15;
      const int k = k0 + kk;
      C a, b;
      a.x = a.y = b.x = b.y = T(0);
      if (k < ke && p0 + r < nproj) a = anl[(size_t)(p0 + r) * lda + k];
      if (k < ke && n0 + r < nst) b = psi[(size_t)(n0 + r) * ld + k];
      As[kk][r] = a;
      Bs[kk][r] = b;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      C a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          ar[i][j] += a[i].x * b[j].x + a[i].y * b[j].y;
          ai[i][j] += a[i].x * b[j].y - a[i].y * b[j].x;
        }
    }
    __syncthreads();
  }
  double2* pz = part + (size_t)blockIdx.z * nst * nproj;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int pp = p0 + ty + 16 * i, nn = n0 + tx + 16 * j;
      if (pp < nproj && nn < nst)
        pz[(size_t)nn * nproj + pp] = make_double2((double)ar[i][j], (double)ai[i][j]);
    }
}

// fnl[n][p] = (D_p/Omega) sum_z part[z][n][p]; enl partials per block
template <typename T>
__global__ void __launch_bounds__(256)
k_fnl_reduce(const double2* __restrict__ part, int nsplit, int nproj, int nst,
             const double* __restrict__ wt, const double* __restrict__ occ,
             cplx<T>* __restrict__ fnl, double* __restrict__ enl_part) {
  __shared__ double red[256];
  const size_t total = (size_t)nproj * nst;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double e = 0.0;
  if (i < total) {
    const int n = (int)(i / nproj), pp = (int)(i - (size_t)n * nproj);
    double re = 0.0, im = 0.0;
    for (int z = 0; z < nsplit; ++z) {
      const double2 v = part[(size_t)z * total + i];
      re += v.x;
      im += v.y;
    }
    const double fac = wt[pp];
    e = (fac * (occ ? occ[n] : 0.0)) * (re * re + im * im);
    cplx<T> f;
    f.x = (T)(fac * re);
    f.y = (T)(fac * im);
    fnl[i] = f;
  }
  red[threadIdx.x] = e;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0 && enl_part) enl_part[blockIdx.x] = red[0];
}

// out[n][g] = sum_p anl[p][g] fnl[n][p], g < ngw; anl rows lda apart
template <typename T>
__global__ void __launch_bounds__(256)
k_nl_hpsi(const cplx<T>* __restrict__ anl, int lda, int ngw, int nproj,
          const cplx<T>* __restrict__ fnl, int nst, cplx<T>* __restrict__ out, int ldo) {
  using C = cplx<T>;
  __shared__ C As[GK][GT];
  __shared__ C Bs[GK][GT];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int g0 = blockIdx.x * GT, n0 = blockIdx.y * GT;
  T ar[4][4], ai[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) ar[i][j] = ai[i][j] = T(0);
  for (int k0 = 0; k0 < nproj; k0 += GK) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = tid + 256 * q;
      {
        const int kk = e >> 6, gg = e & 63;
        C a;
        a.x = a.y = T(0);
        if (k0 + kk < nproj && g0 + gg < ngw) a = anl[(size_t)(k0 + kk) * lda + g0 + gg];
        As[kk][gg] = a;
      }
      {
        const int kk = e & 15, nn = e >> 4;
        C b;
        b.x = b.y = T(0);
        if (k0 + kk < nproj && n0 + nn < nst) b = fnl[(size_t)(n0 + nn) * nproj + k0 + kk];
        Bs[kk][nn] = b;
      }
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      C a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          ar[i][j] += a[i].x * b[j].x - a[i].y * b[j].y;
          ai[i][j] += a[i].x * b[j].y + a[i].y * b[j].x;
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gg = g0 + tx + 16 * i, nn = n0 + ty + 16 * j;
      if (gg < ngw && nn < nst) {
        C o;
        o.x = ar[i][j];
        o.y = ai[i][j];
        out[(size_t)nn * ldo + gg] = o;
      }
    }
}

template <typename T>
qbg_status nl_apply(qbg_plan* p, const cplx<T>* psi, int ld, cplx<T>* out, int nst,
                    const double* d_occ, double* enl_part, cudaStream_t st) {
  const int P = p->nproj;
  if (P == 0 || nst == 0) return QBG_OK;
  const cplx<T>* anl = std::is_same<T, double>::value ? (const cplx<T>*)p->d_anl
                                                       : (const cplx<T>*)p->d_anl32;
  const int mt = (P + GT - 1) / GT, nt = (nst + GT - 1) / GT;
  // split K so that the grid covers the GPU a few times over; FP32 keeps
  // each partial sum short (<= 2048 terms) and adds the partials in FP64
  int nsm = 152;
  int target = 4 * nsm;
  int split = std::max(1, (target + mt * nt - 1) / (mt * nt));
  const int maxk = std::is_same<T, double>::value ? (1 << 30) : 2048;
  split = std::max(split, (p->ngw + maxk - 1) / maxk);
  split = std::min(split, std::max(1, p->ngw / GK));
  int kchunk = (p->ngw + split - 1) / split;
  kchunk = (kchunk + GK - 1) / GK * GK;
  split = (p->ngw + kchunk - 1) / kchunk;
  const size_t need = (size_t)split * P * nst * sizeof(double2);
  qbg_status s = ensure(&p->d_fpart, &p->fpart_bytes, need);
  if (s) return s;
  s = ensure(&p->d_fnl, &p->fnl_bytes, (size_t)P * nst * sizeof(cplx<T>));
  if (s) return s;
  {
    PhaseTimer pt(p, PH_FNL_GEMM, st);
    k_fnl<T><<<dim3(mt, nt, split), 256, 0, st>>>(anl, p->ngw, p->ngw, P, psi, ld, nst,
                                                   (double2*)p->d_fpart, kchunk);
    QBG_LAUNCHED(p);
  }
  const size_t total = (size_t)P * nst;
  const int rb = (int)((total + 255) / 256);
  {
    PhaseTimer pt(p, PH_FNL_REDUCE, st);
    k_fnl_reduce<T><<<rb, 256, 0, st>>>((const double2*)p->d_fpart, split, P, nst, p->d_pwt,
                                        d_occ, (cplx<T>*)p->d_fnl, enl_part);
    QBG_LAUNCHED(p);
  }
  if (p->fnl_export && std::is_same<T, double>::value)
    QBG_CUDA(cudaMemcpyAsync(p->fnl_export, p->d_fnl, sizeof(double2) * total,
                             cudaMemcpyDeviceToDevice, st));
  {
    PhaseTimer pt(p, PH_ENL_HPSI, st);
    k_nl_hpsi<T><<<dim3((p->ngw + GT - 1) / GT, nt), 256, 0, st>>>(
        anl, p->ngw, p->ngw, P, (const cplx<T>*)p->d_fnl, nst, out, ld);
    QBG_LAUNCHED(p);
  }
  return QBG_OK;
}

int nl_reduce_blocks(const qbg_plan* p, int nst) {
  return (int)(((size_t)p->nproj * nst + 255) / 256);
}

template qbg_status nl_apply<double>(qbg_plan*, const double2*, int, double2*, int,
                                     const double*, double*, cudaStream_t);

// ------------------------------------------------- derivative of the table
// dbeta[p][g] = d anl[p][g] / da for A = A0 + a e: the projector k_anl builds
// is kappa_l t(q) exp(-i q.tau) with q = k+G-A, kappa = 1, -i, -1 for
// l = 0, 1, 2 and t = s_l P_lm(q) exp(-|q|^2 rc^2 / 2) (P_lm the solid
// harmonic: 1, q_m, the five quadratics), so with dq/da = -e
//   dbeta = -kappa exp(-i q.tau) (e.grad t - i (e.tau) t),
//   e.grad t = s_l (e.grad P - rc^2 P (e.q)) exp(-|q|^2 rc^2 / 2).
__global__ void __launch_bounds__(256)
k_anl_da(const double* __restrict__ kpgx, const double* __restrict__ kpg2A, int ngw, double A0,
         double A1, double A2, double e0, double e1, double e2, int natoms,
         const AtomDesc* __restrict__ ad, const ProjDesc* __restrict__ pd,
         double2* __restrict__ dbeta) {
  // one thread per G for all atoms: the Y_lm factors and their derivatives
  // along e depend on q = k+G-A only and the radial Gaussian on |q| and the
  // atom's rc (recomputed only when rc changes); per atom the structure
  // phase and the projectors' products remain
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ngw) return;
  const double qx = kpgx[g] - A0, qy = kpgx[ngw + g] - A1, qz = kpgx[2 * ngw + g] - A2;
  const double k2 = kpg2A[g];
  const double eq = e0 * qx + e1 * qy + e2 * qz;
  const double fpi = 4.0 * 3.14159265358979323846;
  const double s3 = sqrt(3.0);
  // (P, eP) of the projector types, index 0 (l = 0), 1 + m (l = 1), 4 + m
  // (l >= 2, m >= 4 sharing the last form)
  const double S0 = sqrt(1.0 / fpi), S1 = sqrt(3.0 / fpi), S2 = sqrt(5.0 / fpi);
  double P[9], eP[9];
  P[0] = 1.0; eP[0] = 0.0;
  P[1] = qx; eP[1] = e0;
  P[2] = qy; eP[2] = e1;
  P[3] = qz; eP[3] = e2;
  P[4] = 0.5 * (2.0 * qz * qz - qx * qx - qy * qy);
  eP[4] = -e0 * qx - e1 * qy + 2.0 * e2 * qz;
  P[5] = 0.5 * s3 * (qx * qx - qy * qy); eP[5] = s3 * (e0 * qx - e1 * qy);
  P[6] = s3 * qx * qy; eP[6] = s3 * (e0 * qy + e1 * qx);
  P[7] = s3 * qy * qz; eP[7] = s3 * (e1 * qz + e2 * qy);
  P[8] = s3 * qx * qz; eP[8] = s3 * (e0 * qz + e2 * qx);
  double rc_prev = -1.0, rc2 = 0.0, E = 0.0;
  for (int ia = 0; ia < natoms; ++ia) {
    const AtomDesc at = ad[ia];
    if (at.rc != rc_prev) {
      rc_prev = at.rc;
      rc2 = at.rc * at.rc;
      E = exp(-0.5 * k2 * rc2);
    }
    const double etau = e0 * at.tau[0] + e1 * at.tau[1] + e2 * at.tau[2];
    double sn, cs;
    sincos(-(at.tau[0] * qx + at.tau[1] * qy + at.tau[2] * qz), &sn, &cs);
    for (int ipr = 0; ipr < at.npr; ++ipr) {
      const int p = at.p0 + ipr * at.stride;
      const int l = pd[p].l, m = pd[p].m;
      const int lm = l == 0 ? 0 : (l == 1 ? 1 + m : 4 + min(m, 4));
      const double sl = l == 0 ? S0 : (l == 1 ? S1 : S2);
      const double t = sl * P[lm] * E;
      const double wr = sl * E * (eP[lm] - rc2 * P[lm] * eq);
      const double wi = -etau * t;
      const double zr = cs * wr - sn * wi, zi = sn * wr + cs * wi;
      double2 o;
      if (l == 0) o = make_double2(-zr, -zi);
      else if (l == 1) o = make_double2(-zi, zr);
      else o = make_double2(zr, zi);
      dbeta[(size_t)p * ngw + g] = o;
    }
  }
}

qbg_status nl_build_da(qbg_plan* p, const double* e, double2* dbeta, cudaStream_t st) {
  if (p->nproj == 0 || p->ngw == 0) return QBG_OK;
  if (p->nl_tables) {
    set_error("projector derivative along A: not available for caller projector tables "
              "(qbg_set_nonlocal_tables carries no radial derivative)");
    return QBG_ERR_UNSUPPORTED;
  }
  if (!p->nl_ready || !p->d_pdesc) {
    set_error("projector derivative: the projector table is not built");
    return QBG_ERR_STATE;
  }
  k_anl_da<<<(p->ngw + 255) / 256, 256, 0, st>>>(
      p->d_kpgx, p->d_kpg2A, p->ngw, p->A[0], p->A[1], p->A[2], e[0], e[1], e[2], p->nl_natoms,
      (const AtomDesc*)p->d_adesc, (const ProjDesc*)p->d_pdesc, dbeta);
  QBG_LAUNCHED(p);
  return QBG_OK;
}

// f[n][p] = sum_z part[z][n][p]
__global__ void k_part_sum(const double2* __restrict__ part, int nsplit, size_t total,
                           double2* __restrict__ f) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  double re = 0.0, im = 0.0;
  for (int z = 0; z < nsplit; ++z) {
    const double2 v = part[(size_t)z * total + i];
    re += v.x;
    im += v.y;
  }
  f[i] = make_double2(re, im);
}

// f[n][p] = sum_g conj(table[p][g]) x[n][g] in FP64 (no weights)
qbg_status nl_project64(qbg_plan* p, const double2* table, const double2* x, int ld, int nst,
                        double2* f, cudaStream_t st) {
  const int P = p->nproj;
  if (P == 0 || nst == 0) return QBG_OK;
  const int mt = (P + GT - 1) / GT, nt = (nst + GT - 1) / GT;
  int split = std::max(1, (4 * 152 + mt * nt - 1) / (mt * nt));
  split = std::min(split, std::max(1, p->ngw / GK));
  int kchunk = (p->ngw + split - 1) / split;
  kchunk = (kchunk + GK - 1) / GK * GK;
  split = (p->ngw + kchunk - 1) / kchunk;
  const qbg_status s = ensure(&p->d_fpart, &p->fpart_bytes, (size_t)split * P * nst * sizeof(double2));
  if (s != QBG_OK) return s;
  k_fnl<double><<<dim3(mt, nt, split), 256, 0, st>>>(table, p->ngw, p->ngw, P, x, ld, nst,
                                                      (double2*)p->d_fpart, kchunk);
  QBG_LAUNCHED(p);
  const size_t total = (size_t)P * nst;
  k_part_sum<<<(unsigned)((total + 255) / 256), 256, 0, st>>>((const double2*)p->d_fpart, split,
                                                              total, f);
  QBG_LAUNCHED(p);
  return QBG_OK;
}

// ---------------------------------------------- Gram (SlaterDet::gram)
// S[n][m] = <psi_m|psi_n> = sum_g conj(psi[m][g]) psi[n][g] (FP64, device)
qbg_status gram_overlap(qbg_plan* p, const double2* psi, int ld, int nst, double2* S,
                        cudaStream_t st) {
  const int mt = (nst + GT - 1) / GT;
  int split = std::max(1, (4 * 152 + mt * mt - 1) / (mt * mt));
  split = std::min(split, std::max(1, p->ngw / GK));
  int kchunk = (p->ngw + split - 1) / split;
  kchunk = (kchunk + GK - 1) / GK * GK;
  split = (p->ngw + kchunk - 1) / kchunk;
  const qbg_status s =
      ensure(&p->d_fpart, &p->fpart_bytes, (size_t)split * nst * nst * sizeof(double2));
  if (s != QBG_OK) return s;
  k_fnl<double><<<dim3(mt, mt, split), 256, 0, st>>>(psi, ld, p->ngw, nst, psi, ld, nst,
                                                      (double2*)p->d_fpart, kchunk);
  QBG_LAUNCHED(p);
  const size_t total = (size_t)nst * nst;
  k_part_sum<<<(unsigned)((total + 255) / 256), 256, 0, st>>>((const double2*)p->d_fpart, split,
                                                              total, S);
  QBG_LAUNCHED(p);
  return QBG_OK;
}

// out[n][g] = sum_m psi[m][g] T[n][m] (FP64, device)
qbg_status gram_apply(qbg_plan* p, const double2* psi, int ld, int nst, const double2* T,
                      double2* out, int ldo, cudaStream_t st) {
  const int nt = (nst + GT - 1) / GT;
  k_nl_hpsi<double><<<dim3((p->ngw + GT - 1) / GT, nt), 256, 0, st>>>(psi, ld, p->ngw, nst, T,
                                                                       nst, out, ldo);
  QBG_LAUNCHED(p);
  return QBG_OK;
}

}  // namespace qbg
