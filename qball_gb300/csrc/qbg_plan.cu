// qbg_plan.cu -- error reporting, basis construction, transform tables and
// plan life cycle.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <string>
#include <vector>

#include "qbg_internal.h"

namespace qbg {

static thread_local std::string g_err;

const char* const kPhaseName[PH_COUNT] = {
    "fnl_gemm", "fnl_reduce", "enl_hpsi", "ft_z_bwd", "ft_x_bwd", "ft_y_vloc",
    "ft_x_fwd", "ft_z_fwd", "ft_y_density", "ft_y_store", "ft_y_load", "misc", "ft_xyx_vloc",
    "ft_xy_pair"};

void set_error(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
}

qbg_status cuda_status(cudaError_t e, const char* what) {
  set_error("CUDA error in %s: %s", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? QBG_ERR_NOMEM : QBG_ERR_CUDA;
}

qbg_status ensure(void** p, size_t* cur, size_t need) {
  if (need <= *cur && *p) return QBG_OK;
  if (*p) {
    // the old buffer may still be read by queued kernels
    cudaDeviceSynchronize();
    cudaFree(*p);
  }
  *p = nullptr;
  *cur = 0;
  if (need == 0) return QBG_OK;
  cudaError_t e = cudaMalloc(p, need);
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_status(e, "cudaMalloc (scratch)");
  }
  *cur = need;
  return QBG_OK;
}

qbg_status ensure_host(double** p, size_t* cur, size_t need) {
  if (need <= *cur && *p) return QBG_OK;
  if (*p) cudaFreeHost(*p);
  *p = nullptr;
  *cur = 0;
  cudaError_t e = cudaMallocHost((void**)p, need);
  if (e != cudaSuccess) return cuda_status(e, "cudaMallocHost");
  *cur = need;
  return QBG_OK;
}

// ------------------------------------------------------------------ basis
// Full-sphere plane-wave basis at k=0 on one process.  The construction
// follows Basis::resize (Basis.cc:302-700): rods (h,k) of the lattice points
// with |G|^2 < 2 ecut, scanned h outer / k inner over the safe enclosing box,
// kept in ascending rod length with ties in scan order (the reference's
// multiset<Rod>), then rod (0,0) exchanged with the first rod.  The lattice
// arithmetic reproduces UnitCell::set (UnitCell.cc:37-80) and D3vector
// operation by operation, so G vectors and |G|^2 are bit-identical.
namespace {
struct Rod {
  int h, k, lmin, size;
};

void cell_b(const double* a, double* b, double* vol) {
  auto cross = [](const double* x, const double* y, double* z) {
    z[0] = x[1] * y[2] - x[2] * y[1];
    z[1] = x[2] * y[0] - x[0] * y[2];
    z[2] = x[0] * y[1] - x[1] * y[0];
  };
  double c[3];
  cross(a + 3, a + 6, c);
  // host code is built with -ffp-contract=off: every product is rounded
  *vol = a[0] * c[0] + a[1] * c[1] + a[2] * c[2];
  if (!(*vol > 0.0)) {
    std::memset(b, 0, 9 * sizeof(double));
    return;
  }
  const double fac = 1.0 / *vol;
  const double twopi = 2.0 * M_PI;
  for (int i = 0; i < 3; ++i) {
    const double* p = a + 3 * ((i + 1) % 3);
    const double* q = a + 3 * ((i + 2) % 3);
    double fp[3] = {p[0] * fac, p[1] * fac, p[2] * fac};
    double z[3];
    cross(fp, q, z);
    for (int j = 0; j < 3; ++j) b[3 * i + j] = z[j] * twopi;
  }
}

bool fft_friendly(int n) {
  // ESSL-style lengths accepted by Basis::factorizable (Basis.cc:126-150)
  if (n % 11 == 0) n /= 11;
  if (n % 7 == 0) n /= 7;
  if (n % 5 == 0) n /= 5;
  if (n % 3 == 0) n /= 3;
  if (n % 3 == 0) n /= 3;
  while (n % 2 == 0) n /= 2;
  return n == 1;
}

std::vector<Rod> build_rods(const double* a, double ecut, int* info) {
  double b[9], vol;
  cell_b(a, b, &vol);
  const double two_ecut = 2.0 * ecut;
  const double fac = std::sqrt(two_ecut) / (2.0 * M_PI);
  auto len = [](const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); };
  const int hmax = (int)(0.5 + fac * len(a)), kmax = (int)(0.5 + fac * len(a + 3));
  const int lmax = (int)(0.5 + fac * len(a + 6));
  const int hmin = -hmax, kmin = -kmax, lmin = -lmax;
  std::vector<Rod> rods;
  int used[6] = {hmin, hmax, kmin, kmax, lmin, lmax};  // max_h,min_h,max_k,min_k,max_l,min_l
  int size = 0;
  for (int h = hmin - 1; h <= hmax + 1; ++h) {
    for (int k = kmin - 1; k <= kmax + 1; ++k) {
      int lstart = lmax, lend = lmin;
      bool found = false;
      for (int l = lmin - 1; l <= lmax + 1; ++l) {
        double v[3];
        for (int j = 0; j < 3; ++j)
          v[j] = (b[j] * (0.0 + h) + b[3 + j] * (0.0 + k)) + b[6 + j] * (0.0 + l);
        const double two_e = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        if (two_e < two_ecut) {
          lstart = std::min(l, lstart);
          lend = std::max(l, lend);
          found = true;
        }
      }
      if (found) {
        rods.push_back({h, k, lstart, lend - lstart + 1});
        size += lend - lstart + 1;
        used[0] = std::max(h, used[0]);
        used[1] = std::min(h, used[1]);
        used[2] = std::max(k, used[2]);
        used[3] = std::min(k, used[3]);
        used[4] = std::max(lend, used[4]);
        used[5] = std::min(lstart, used[5]);
      }
    }
  }
  std::stable_sort(rods.begin(), rods.end(),
                   [](const Rod& x, const Rod& y) { return x.size < y.size; });
  for (size_t i = 0; i < rods.size(); ++i)
    if (rods[i].h == 0 && rods[i].k == 0) {
      std::swap(rods[0], rods[i]);
      break;
    }
  const int mx[3] = {hmax, kmax, lmax};
  int np[3];
  for (int i = 0; i < 3; ++i) {
    int n = 2 * mx[i] + 2;
    while (!fft_friendly(n)) n += 2;
    np[i] = n;
  }
  if (info) {
    info[0] = size;
    info[1] = (int)rods.size();
    info[2] = np[0];
    info[3] = np[1];
    info[4] = np[2];
    info[5] = used[1];
    info[6] = used[3];
    info[7] = used[5];
    info[8] = used[0];
    info[9] = used[2];
    info[10] = used[4];
    info[11] = 0;
  }
  return rods;
}

// ------------------------------------------------------- transform tables
// Radices with a hand-written codelet (7, 11, 13 are direct DFTs).
bool is_codelet(int r) {
  switch (r) {
    case 2: case 3: case 4: case 5: case 6: case 7: case 8: case 9:
    case 10: case 11: case 12: case 13: case 15: case 16: return true;
    default: return false;
  }
}

// Radix orders of the Stockham passes (the autotuner's choice):
//   0: greedy 8/4/2, then the odd primes (default);
//   1: the odd primes first, then 8/4/2;
//   2: radix 4 preferred (4s, then 2), then the odd primes.
// (Two-pass splits with the 9..16-point codelets were measured slower on
// GB300: the larger codelets raise the register count of every transform
// kernel and cut its occupancy.)
bool factorize(int n, LenTables& L, int order) {
  int r[16], np = 0;
  {
    int m = n;
    auto odd = [&]() {
      for (int q : {3, 5, 7, 11, 13})
        while (m % q == 0 && np < 16) { r[np++] = q; m /= q; }
    };
    auto pow2 = [&]() {
      if (order == 2) {
        while (m % 4 == 0 && m > 1 && np < 16) { r[np++] = 4; m /= 4; }
      } else {
        while (m % 8 == 0 && m > 1 && np < 16) { r[np++] = 8; m /= 8; }
        if (m % 4 == 0) { r[np++] = 4; m /= 4; }
      }
      if (m % 2 == 0) { r[np++] = 2; m /= 2; }
    };
    if (order == 1) {
      odd();
      pow2();
    } else {
      pow2();
      odd();
    }
    if (m != 1) return false;
  }
  if (np > kMaxPass) return false;
  L.n = n;
  L.npass = np;
  int ns = 1, off = 0;
  for (int p = 0; p < np; ++p) {
    L.radix[p] = r[p];
    L.ns[p] = ns;
    L.twoff[p] = off;
    off += ns * r[p];
    ns *= r[p];
  }
  return true;
}

// exp(-2 pi i t / M) in long double, t reduced mod M
void unit_root(long long t, long long M, double* re, double* im) {
  t %= M;
  const long double pi = 3.14159265358979323846264338327950288L;
  const long double ang = 2.0L * pi * (long double)t / (long double)M;
  *re = (double)std::cos(ang);
  *im = (double)-std::sin(ang);
}

qbg_status build_len(int n, LenTables& L, int order) {
  if (!factorize(n, L, order)) {
    set_error("grid length %d has a prime factor outside {2,3,5,7,11,13} or too many passes", n);
    return QBG_ERR_UNSUPPORTED;
  }
  int ntw = 0;
  for (int p = 0; p < L.npass; ++p) ntw += L.ns[p] * L.radix[p];
  L.ntw = ntw;
  std::vector<double2> tw(ntw);
  for (int p = 0; p < L.npass; ++p) {
    const int R = L.radix[p], Ns = L.ns[p];
    for (int k = 0; k < Ns; ++k)
      for (int r = 0; r < R; ++r) {
        double c, s;
        unit_root((long long)r * k, (long long)Ns * R, &c, &s);
        tw[L.twoff[p] + k * R + r] = make_double2(c, s);
      }
  }
  std::vector<double2> g(7 + 11 + 13);
  L.goff7 = 0;
  L.goff11 = 7;
  L.goff13 = 18;
  for (int m = 0; m < 7; ++m) unit_root(m, 7, &g[m].x, &g[m].y);
  for (int m = 0; m < 11; ++m) unit_root(m, 11, &g[7 + m].x, &g[7 + m].y);
  for (int m = 0; m < 13; ++m) unit_root(m, 13, &g[18 + m].x, &g[18 + m].y);
  std::vector<float2> tw32(ntw), g32(g.size());
  for (int i = 0; i < ntw; ++i) tw32[i] = make_float2((float)tw[i].x, (float)tw[i].y);
  for (size_t i = 0; i < g.size(); ++i) g32[i] = make_float2((float)g[i].x, (float)g[i].y);
  // double-float tables from the extended-precision values
  auto to_df = [](long double v) {
    const float h = (float)v;
    return df32(h, (float)(v - (long double)h));
  };
  std::vector<df32c> twdf(ntw), gdf(g.size());
  for (int p = 0; p < L.npass; ++p) {
    const int R = L.radix[p], Ns = L.ns[p];
    for (int k = 0; k < Ns; ++k)
      for (int r = 0; r < R; ++r) {
        const long long t = ((long long)r * k) % ((long long)Ns * R);
        const long double pi = 3.14159265358979323846264338327950288L;
        const long double ang = 2.0L * pi * (long double)t / (long double)(Ns * R);
        twdf[L.twoff[p] + k * R + r] = df32c{to_df(std::cos(ang)), to_df(-std::sin(ang))};
      }
  }
  {
    const int ps[3] = {7, 11, 13}, off[3] = {0, 7, 18};
    for (int q = 0; q < 3; ++q)
      for (int m = 0; m < ps[q]; ++m) {
        const long double pi = 3.14159265358979323846264338327950288L;
        const long double ang = 2.0L * pi * (long double)m / (long double)ps[q];
        gdf[off[q] + m] = df32c{to_df(std::cos(ang)), to_df(-std::sin(ang))};
      }
  }
  {
    std::vector<double2> r64(n);
    std::vector<float2> r32(n);
    std::vector<df32c> rdf(n);
    for (int m = 0; m < n; ++m) {
      const long double pi = 3.14159265358979323846264338327950288L;
      const long double ang = 2.0L * pi * (long double)m / (long double)n;
      const long double c = std::cos(ang), sn = -std::sin(ang);
      r64[m] = make_double2((double)c, (double)sn);
      r32[m] = make_float2((float)c, (float)sn);
      rdf[m] = df32c{to_df(c), to_df(sn)};
    }
    QBG_CUDA(cudaMalloc(&L.d_root64, sizeof(double2) * n));
    QBG_CUDA(cudaMalloc(&L.d_root32, sizeof(float2) * n));
    QBG_CUDA(cudaMalloc(&L.d_rootdf, sizeof(df32c) * n));
    QBG_CUDA(cudaMemcpy(L.d_root64, r64.data(), sizeof(double2) * n, cudaMemcpyHostToDevice));
    QBG_CUDA(cudaMemcpy(L.d_root32, r32.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
    QBG_CUDA(cudaMemcpy(L.d_rootdf, rdf.data(), sizeof(df32c) * n, cudaMemcpyHostToDevice));
  }
  QBG_CUDA(cudaMalloc(&L.d_twdf, sizeof(df32c) * ntw));
  QBG_CUDA(cudaMalloc(&L.d_gdf, sizeof(df32c) * gdf.size()));
  QBG_CUDA(cudaMemcpy(L.d_twdf, twdf.data(), sizeof(df32c) * ntw, cudaMemcpyHostToDevice));
  QBG_CUDA(cudaMemcpy(L.d_gdf, gdf.data(), sizeof(df32c) * gdf.size(), cudaMemcpyHostToDevice));
  QBG_CUDA(cudaMalloc(&L.d_tw64, sizeof(double2) * ntw));
  QBG_CUDA(cudaMalloc(&L.d_tw32, sizeof(float2) * ntw));
  QBG_CUDA(cudaMalloc(&L.d_g64, sizeof(double2) * g.size()));
  QBG_CUDA(cudaMalloc(&L.d_g32, sizeof(float2) * g.size()));
  QBG_CUDA(cudaMemcpy(L.d_tw64, tw.data(), sizeof(double2) * ntw, cudaMemcpyHostToDevice));
  QBG_CUDA(cudaMemcpy(L.d_tw32, tw32.data(), sizeof(float2) * ntw, cudaMemcpyHostToDevice));
  QBG_CUDA(cudaMemcpy(L.d_g64, g.data(), sizeof(double2) * g.size(), cudaMemcpyHostToDevice));
  QBG_CUDA(cudaMemcpy(L.d_g32, g32.data(), sizeof(float2) * g.size(), cudaMemcpyHostToDevice));
  return QBG_OK;
}

void free_len(LenTables& L) {
  cudaFree(L.d_tw64);
  cudaFree(L.d_tw32);
  cudaFree(L.d_g64);
  cudaFree(L.d_g32);
  cudaFree(L.d_twdf);
  cudaFree(L.d_gdf);
  cudaFree(L.d_root64);
  cudaFree(L.d_root32);
  cudaFree(L.d_rootdf);
  L.d_twdf = nullptr;
  L.d_gdf = nullptr;
  L.d_root64 = nullptr;
  L.d_root32 = nullptr;
  L.d_rootdf = nullptr;
  L.d_tw64 = nullptr;
  L.d_tw32 = nullptr;
  L.d_g64 = nullptr;
  L.d_g32 = nullptr;
}

template <typename D, typename S> qbg_status upload(D** d, const S* h, size_t n) {
  QBG_CUDA(cudaMalloc(d, sizeof(D) * (n ? n : 1)));
  if (n) QBG_CUDA(cudaMemcpy(*d, h, sizeof(D) * n, cudaMemcpyHostToDevice));
  return QBG_OK;
}
}  // namespace

template <> FFTLen<double> LenTables::view<double>() const {
  FFTLen<double> d;
  d.n = n;
  d.npass = npass;
  d.ntw = ntw;
  for (int i = 0; i < kMaxPass; ++i) {
    d.radix[i] = radix[i];
    d.ns[i] = ns[i];
    d.twoff[i] = twoff[i];
    d.inv_m[i] = radix[i] ? 1.0f / (float)(n / radix[i]) : 0.f;
    d.inv_ns[i] = ns[i] ? 1.0f / (float)ns[i] : 0.f;
  }
  d.tw = d_tw64;
  d.gtab = d_g64;
  d.root = d_root64;
  d.goff7 = goff7;
  d.goff11 = goff11;
  d.goff13 = goff13;
  d.pfa = allow_pfa ? pfa_split(n) : 0;
  return d;
}
template <> FFTLen<df32> LenTables::view<df32>() const {
  FFTLen<df32> d;
  d.n = n;
  d.npass = npass;
  d.ntw = ntw;
  for (int i = 0; i < kMaxPass; ++i) {
    d.radix[i] = radix[i];
    d.ns[i] = ns[i];
    d.twoff[i] = twoff[i];
    d.inv_m[i] = radix[i] ? 1.0f / (float)(n / radix[i]) : 0.f;
    d.inv_ns[i] = ns[i] ? 1.0f / (float)ns[i] : 0.f;
  }
  d.tw = d_twdf;
  d.gtab = d_gdf;
  d.root = d_rootdf;
  d.goff7 = goff7;
  d.goff11 = goff11;
  d.goff13 = goff13;
  d.pfa = allow_pfa ? pfa_split(n) : 0;
  return d;
}
template <> FFTLen<float> LenTables::view<float>() const {
  FFTLen<float> d;
  d.n = n;
  d.npass = npass;
  d.ntw = ntw;
  for (int i = 0; i < kMaxPass; ++i) {
    d.radix[i] = radix[i];
    d.ns[i] = ns[i];
    d.twoff[i] = twoff[i];
    d.inv_m[i] = radix[i] ? 1.0f / (float)(n / radix[i]) : 0.f;
    d.inv_ns[i] = ns[i] ? 1.0f / (float)ns[i] : 0.f;
  }
  d.tw = d_tw32;
  d.gtab = d_g32;
  d.root = d_root32;
  d.goff7 = goff7;
  d.goff11 = goff11;
  d.goff13 = goff13;
  d.pfa = allow_pfa ? pfa_split(n) : 0;
  return d;
}

}  // namespace qbg

using namespace qbg;

extern "C" {

const char* qbg_last_error(void) { return g_err.c_str(); }
const char* qbg_version(void) { return "qball-gb300 0.1 (sm_103a)"; }

// a right-handed cell of positive volume (UnitCell::volume() > 0)
static bool cell_ok(const double* a) {
  double b[9], vol;
  cell_b(a, b, &vol);
  return vol > 0.0 && std::isfinite(vol);
}

qbg_status qbg_basis_dims(const double* a, double ecut, int* info) {
  if (!a || !info || !(ecut >= 0.0)) {
    set_error("qbg_basis_dims: null argument or negative ecut");
    return QBG_ERR_INVALID;
  }
  if (!cell_ok(a)) {
    set_error("qbg_basis_dims: the cell vectors span no positive volume");
    return QBG_ERR_INVALID;
  }
  build_rods(a, ecut, info);
  return QBG_OK;
}

qbg_status qbg_basis_fill(const double* a, double ecut, int* rod_h, int* rod_k,
                          int* rod_lmin, int* rod_size, int* idx, double* kpg2,
                          double* kpgx) {
  if (!a || !(ecut >= 0.0)) {
    set_error("qbg_basis_fill: null cell or negative ecut");
    return QBG_ERR_INVALID;
  }
  if (!cell_ok(a)) {
    set_error("qbg_basis_fill: the cell vectors span no positive volume");
    return QBG_ERR_INVALID;
  }
  int info[12];
  std::vector<Rod> rods = build_rods(a, ecut, info);
  const int ng = info[0];
  double b[9], vol;
  cell_b(a, b, &vol);
  int i = 0;
  for (size_t r = 0; r < rods.size(); ++r) {
    if (rod_h) rod_h[r] = rods[r].h;
    if (rod_k) rod_k[r] = rods[r].k;
    if (rod_lmin) rod_lmin[r] = rods[r].lmin;
    if (rod_size) rod_size[r] = rods[r].size;
    for (int l = 0; l < rods[r].size; ++l, ++i) {
      const int ih = rods[r].h, ik = rods[r].k, il = rods[r].lmin + l;
      if (idx) {
        idx[3 * i] = ih;
        idx[3 * i + 1] = ik;
        idx[3 * i + 2] = il;
      }
      // Basis::update_g (Basis.cc:700-735)
      double v[3];
      for (int j = 0; j < 3; ++j)
        v[j] = (b[j] * (0.0 + ih) + b[3 + j] * (0.0 + ik)) + b[6 + j] * (0.0 + il);
      if (kpgx) {
        kpgx[i] = v[0];
        kpgx[ng + i] = v[1];
        kpgx[2 * ng + i] = v[2];
      }
      if (kpg2) kpg2[i] = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    }
  }
  return QBG_OK;
}

qbg_status qbg_plan_destroy(qbg_plan* p) {
  if (!p) return QBG_OK;
  adj_release(p);
  tc_release(p);
  oz_release(p);
  hxc_release(p);
  for (auto& L : p->len) free_len(L);
  void* bufs[] = {p->d_rods, p->d_row_ptr, p->d_row_rod, p->d_row_x, p->d_band_y,
                  p->d_kpgx, p->d_kpg2A, p->d_kpg2A32, p->d_vr, p->d_vr32, p->d_vrdf,
                  p->d_plist, p->d_ptau, p->d_pwt, p->d_pl, p->d_prc, p->d_pdesc, p->d_adesc,
                  p->d_anl, p->d_anl32, p->d_twnl, p->d_vhist, p->d_Z, p->d_Y, p->d_fnl,
                  p->d_fpart,
                  p->d_red, p->d_rho, p->d_rho_slots, p->d_vsph, p->d_w[0], p->d_w[1], p->d_w[2], p->d_w[3]};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (p->h_red) cudaFreeHost(p->h_red);
  delete p;
  return QBG_OK;
}

qbg_status qbg_plan_create(const qbg_basis_desc* bd, int np0, int np1, int np2,
                           int precision, qbg_plan** out) {
  if (!bd || !out || bd->ngw < 0 || bd->nrods < 0 || np0 <= 0 || np1 <= 0 || np2 <= 0 ||
      (bd->ngw > 0 && (!bd->rod_h || !bd->rod_k || !bd->rod_lmin || !bd->rod_size || !bd->kpgx)) ||
      precision < QBG_PREC_FP64 || precision > QBG_PREC_MIXED_DF32 || !(bd->omega > 0.0)) {
    set_error("qbg_plan_create: invalid argument");
    return QBG_ERR_INVALID;
  }
  if ((long long)np0 * np1 * np2 > (1LL << 31) - 1) {
    set_error("qbg_plan_create: grid too large");
    return QBG_ERR_INVALID;
  }
  *out = nullptr;
  qbg_plan* p = new qbg_plan;
  p->prec = precision;
  p->ngw = bd->ngw;
  p->nrods = bd->nrods;
  p->np0 = np0;
  p->np1 = np1;
  p->np2 = np2;
  p->N = (long long)np0 * np1 * np2;
  p->omega = bd->omega;
  p->rod_h.assign(bd->rod_h, bd->rod_h + bd->nrods);
  p->rod_k.assign(bd->rod_k, bd->rod_k + bd->nrods);
  p->rod_lmin.assign(bd->rod_lmin, bd->rod_lmin + bd->nrods);
  p->rod_size.assign(bd->rod_size, bd->rod_size + bd->nrods);
  p->kpgx_host.assign(bd->kpgx, bd->kpgx + 3 * (size_t)bd->ngw);

  // ntrans0 = max |k| + 1 over the basis (FourierTransform.cc:200-203)
  int kabs = 0, hmin = 0, hmax = 0, lmin = 0, lmax = 0, tot = 0;
  for (int r = 0; r < p->nrods; ++r) {
    kabs = std::max(kabs, std::abs(p->rod_k[r]));
    hmin = std::min(hmin, p->rod_h[r]);
    hmax = std::max(hmax, p->rod_h[r]);
    lmin = std::min(lmin, p->rod_lmin[r]);
    lmax = std::max(lmax, p->rod_lmin[r] + p->rod_size[r] - 1);
    if (p->rod_size[r] <= 0) {
      set_error("qbg_plan_create: rod %d has non-positive size", r);
      qbg_plan_destroy(p);
      return QBG_ERR_INVALID;
    }
    tot += p->rod_size[r];
  }
  if (tot != p->ngw) {
    set_error("qbg_plan_create: rod sizes sum to %d, ngw is %d", tot, p->ngw);
    qbg_plan_destroy(p);
    return QBG_ERR_INVALID;
  }
  p->ntrans0 = kabs + 1;
  p->nband = 2 * p->ntrans0;
  if (p->nband > np1 || hmax - hmin >= np0 || lmax - lmin >= np2) {
    set_error("qbg_plan_create: grid %dx%dx%d too small for the basis (needs np1 >= %d)",
              np0, np1, np2, p->nband);
    qbg_plan_destroy(p);
    return QBG_ERR_INVALID;
  }
  const int ns[3] = {np0, np1, np2};
  for (int d = 0; d < 3; ++d) {
    qbg_status s = build_len(ns[d], p->len[d], 0);
    if (s != QBG_OK) {
      qbg_plan_destroy(p);
      return s;
    }
  }
  // rod and band-row tables
  std::vector<RodInfo> ri(p->nrods);
  std::vector<int> cnt(p->nband + 1, 0);
  int first = 0;
  auto band_of = [&](int k) { return k >= 0 ? k : k + p->nband; };
  for (int r = 0; r < p->nrods; ++r) {
    const int x = ((p->rod_h[r] % np0) + np0) % np0;
    const int b = band_of(p->rod_k[r]);
    ri[r] = {first, p->rod_size[r], p->rod_lmin[r], x | (b << 16)};
    first += p->rod_size[r];
    cnt[b + 1]++;
  }
  for (int b = 0; b < p->nband; ++b) cnt[b + 1] += cnt[b];
  std::vector<int> row_rod(p->nrods), row_x(p->nrods), fill(cnt.begin(), cnt.end() - 1);
  for (int r = 0; r < p->nrods; ++r) {
    const int b = ri[r].xb >> 16;
    row_rod[fill[b]] = r;
    row_x[fill[b]] = ri[r].xb;  // x | band << 16
    fill[b]++;
  }
  std::vector<int> band_y(p->nband);
  for (int b = 0; b < p->nband; ++b) band_y[b] = b < p->ntrans0 ? b : b - p->nband + np1;
  std::vector<double> kpg2(p->ngw);
  std::vector<float> kpg2f(p->ngw);
  const size_t ng = p->ngw;
  for (size_t i = 0; i < ng; ++i) {
    const double kx = p->kpgx_host[i], ky = p->kpgx_host[ng + i], kz = p->kpgx_host[2 * ng + i];
    kpg2[i] = kx * kx + ky * ky + kz * kz;
    kpg2f[i] = (float)kpg2[i];
  }
  qbg_status s = QBG_OK;
  if ((s = upload(&p->d_rods, ri.data(), ri.size())) ||
      (s = upload(&p->d_row_ptr, cnt.data(), cnt.size())) ||
      (s = upload(&p->d_row_rod, row_rod.data(), row_rod.size())) ||
      (s = upload(&p->d_row_x, row_x.data(), row_x.size())) ||
      (s = upload(&p->d_band_y, band_y.data(), band_y.size())) ||
      (s = upload(&p->d_kpgx, p->kpgx_host.data(), p->kpgx_host.size())) ||
      (s = upload(&p->d_kpg2A, kpg2.data(), kpg2.size())) ||
      (s = upload(&p->d_kpg2A32, kpg2f.data(), kpg2f.size()))) {
    qbg_plan_destroy(p);
    return s;
  }
  cudaError_t e = cudaMalloc(&p->d_vr, sizeof(double) * p->N);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_vr32, sizeof(float) * p->N);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_vrdf, sizeof(df32) * p->N);
  if (e == cudaSuccess) e = cudaMemset(p->d_vrdf, 0, sizeof(df32) * p->N);
  if (e == cudaSuccess) e = cudaMemset(p->d_vr, 0, sizeof(double) * p->N);
  if (e == cudaSuccess) e = cudaMemset(p->d_vr32, 0, sizeof(float) * p->N);
  if (e != cudaSuccess) {
    qbg_status st = cuda_status(e, "qbg_plan_create");
    qbg_plan_destroy(p);
    return st;
  }
  // states per transform launch group: 96 on 120 x 120 planes, where the
  // persistent whole-plane kernels gain from longer item lists (28.1 ms per
  // H|psi> of the 216-atom cell against 28.8 ms at 32), else 32
  p->chunk = (np0 == 120 && np1 == 120) ? 96 : 32;
  *out = p;
  return QBG_OK;
}

qbg_status qbg_plan_set_chunk(qbg_plan* p, int states) {
  if (!p || states < 1 || states > 65535) {
    set_error("qbg_plan_set_chunk: invalid argument");
    return QBG_ERR_INVALID;
  }
  p->chunk = states;
  return QBG_OK;
}

qbg_status qbg_plan_set_transform_config(qbg_plan* p, int radix_order, int prime_factor,
                                         int fused, int lane_group) {
  if (!p || radix_order < 0 || radix_order > 2 || fused < 0 || fused > 2) {
    set_error("qbg_plan_set_transform_config: radix_order and fused must be 0, 1 or 2");
    return QBG_ERR_INVALID;
  }
  if (radix_order != p->radix_order) {
    QBG_CUDA(cudaDeviceSynchronize());  // kernels may still read the old tables
    const int ns[3] = {p->np0, p->np1, p->np2};
    for (int d = 0; d < 3; ++d) {
      LenTables L;
      qbg_status s = build_len(ns[d], L, radix_order);
      if (s != QBG_OK) {
        free_len(L);
        return s;
      }
      free_len(p->len[d]);
      p->len[d] = L;
    }
    p->radix_order = radix_order;
  }
  for (auto& L : p->len) L.allow_pfa = prime_factor != 0;
  p->fuse_xyx = fused != 0;
  p->plane_xyx = fused == 2;
  p->lane_fft = lane_group != 0;
  return QBG_OK;
}

qbg_status qbg_plan_get_transform_config(const qbg_plan* p, int* cfg) {
  if (!p || !cfg) {
    set_error("qbg_plan_get_transform_config: null argument");
    return QBG_ERR_INVALID;
  }
  cfg[0] = p->chunk;
  cfg[1] = p->radix_order;
  cfg[2] = p->len[0].allow_pfa ? 1 : 0;
  cfg[3] = p->fuse_xyx ? (p->plane_xyx ? 2 : 1) : 0;
  cfg[4] = p->lane_fft ? 1 : 0;
  return QBG_OK;
}

qbg_status qbg_plan_set_fp64_gemm(qbg_plan* p, int mode, int slices) {
  if (!p || (mode != QBG_GEMM_SIMT && mode != QBG_GEMM_OZAKI) ||
      (mode == QBG_GEMM_OZAKI && slices != 6 && slices != 7)) {
    set_error("qbg_plan_set_fp64_gemm: mode must be QBG_GEMM_SIMT or QBG_GEMM_OZAKI with 6 or "
              "7 slices");
    return QBG_ERR_INVALID;
  }
  if (mode != p->fp64_gemm || (mode == QBG_GEMM_OZAKI && slices != p->oz_slices)) {
    QBG_CUDA(cudaDeviceSynchronize());  // kernels may still read the old slices
    oz_release(p);
  }
  p->fp64_gemm = mode;
  if (mode == QBG_GEMM_OZAKI) p->oz_slices = slices;
  return QBG_OK;
}

qbg_status qbg_plan_set_wait_polls(qbg_plan* p, int polls) {
  if (!p || polls < -1 || polls > (1 << 21)) {
    set_error("qbg_plan_set_wait_polls: polls must be -1 (default) or in [0, 2^21]");
    return QBG_ERR_INVALID;
  }
  p->tc_polls = polls;
  return QBG_OK;
}

qbg_status qbg_profile(qbg_plan* p, int enable) {
  if (!p) {
    set_error("qbg_profile: null plan");
    return QBG_ERR_INVALID;
  }
  p->prof = enable != 0;
  for (int i = 0; i < PH_COUNT; ++i) {
    p->prof_ms[i] = 0.0;
    p->prof_n[i] = 0;
  }
  return QBG_OK;
}

qbg_status qbg_profile_read(const qbg_plan* p, double* ms, long long* launches, int n) {
  if (!p || n < 0 || (n > 0 && (!ms || !launches))) {
    set_error("qbg_profile_read: invalid argument");
    return QBG_ERR_INVALID;
  }
  for (int i = 0; i < n && i < PH_COUNT; ++i) {
    ms[i] = p->prof_ms[i];
    launches[i] = p->prof_n[i];
  }
  return QBG_OK;
}

const char* qbg_phase_name(int i) { return (i >= 0 && i < PH_COUNT) ? kPhaseName[i] : ""; }

qbg_status qbg_launch_count(const qbg_plan* p, long long* count) {
  if (!p || !count) {
    set_error("qbg_launch_count: null argument");
    return QBG_ERR_INVALID;
  }
  *count = p->launches + (p->vplan ? p->vplan->launches : 0);
  return QBG_OK;
}

}  // extern "C"
