// qbg_fft.cu -- sphere <-> grid transforms and the fused local-potential and
// density passes.
//
// One state's 3-D transform is split the way the reference splits it
// (FourierTransform.cc:584-1360), without its MPI transpose:
//   z pass : one line per rod (h,k); the rod's coefficients are gathered from
//            the sphere straight into the line (vector_to_zvec fused), the
//            result written plane-major Z[z][rod] so the next pass reads one
//            contiguous row of rods per plane;
//   x pass : one line per band row (the 2*ntrans0 rows y in [0,ntrans0) and
//            [np1-ntrans0,np1) that can be non-zero), Y[z][band][x];
//   y pass : one line per column x of a plane, where the pointwise work is
//            fused: v(r)*psi(r) between the backward and forward transform
//            (SlaterDet::rs_mul_add), |psi|^2 accumulation (compute_density),
//            or the store of the full grid (plain backward).
// The forward direction runs the same passes in reverse and fuses the
// sphere scatter, the 1/N scale, the kinetic term and the Taylor-series
// accumulation into the last z pass.  On 120 x 120 planes the x and y passes
// run as one whole-plane kernel per (plane, state) item (qbg_plane.cu); the
// band-row fused kernels below serve the 48 and 40 grids, and the separate
// x and y passes every other grid.
// States are processed in chunks (launch groups) that bound the Z/Y
// intermediates.
#include <algorithm>

#include "qbg_internal.h"
#include "qbg_lanefft.cuh"

namespace qbg {

constexpr int kTile = 16;     // lines per CTA
constexpr int kThreads = 256;
// rods per CTA of the forward z pass on 120-point lines (kThreads
// threads): the in-place passes' 40, 24 and 15 items per line come to 5, 3
// and 1.875 rounds per thread
constexpr int kTileZ120 = 32;
// rods a warp gathers at once in the backward z pass: 2 keeps the kernel
// at 64 registers (28 resident warps per SM instead of 15 at 4 rods and
// 110 registers); 1.54 ms per H|psi> of the 216-atom cell against 1.74
#ifndef QBG_ZGATHER_RODS
#define QBG_ZGATHER_RODS 2
#endif
constexpr int kZGather = QBG_ZGATHER_RODS;

// shared-memory elements (complex T) ahead of any v tile: one line buffer
// when the prime-factor transform runs in place, else two plus the twiddles
template <typename T>
__host__ __device__ __forceinline__ int fft_smem_elems(const FFTLen<T>& d, int threads) {
  const int ls = d.n + 1;
  if (d.pfa && kTile * d.pfa <= threads) return kTile * ls;
  return 2 * kTile * ls + d.ntw + kGtab;
}

template <int BYTES>
__device__ __forceinline__ void cp_async(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(d), "l"(src), "n"(BYTES));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <typename T> __device__ __forceinline__ T from_f64(double x) { return (T)x; }
template <> __device__ __forceinline__ df32 from_f64<df32>(double x) { return df32_from_f64(x); }

template <typename T> __device__ __forceinline__ cplx<T> czero() {
  cplx<T> c;
  c.x = T(0);
  c.y = T(0);
  return c;
}

// ------------------------------------------------------------------ z pass
// backward: gather rods of state blockIdx.y from the sphere, transform
// along z, write Z[s][z][rod].
template <typename T, bool BIGP, bool L120 = false>
__global__ void __launch_bounds__(kThreads)
k_z_bwd(const double2* __restrict__ psi, int ld, cplx<T>* __restrict__ Z,
        const RodInfo* __restrict__ rods, int nrods, FFTLen<T> d) {
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem[];
  const int n2 = d.n, ls = n2 + 1;
  C* A = reinterpret_cast<C*>(smem);
  constexpr int TILE = kTile;
  C* B = A + TILE * ls;
  const FFTLen<T> dv = stage_twiddles<T>(d, B + TILE * ls, BIGP);
  const int r0 = blockIdx.x * TILE;
  const int nl = min(TILE, nrods - r0);
  const double2* ps = psi + (size_t)blockIdx.y * ld;
  for (int i = threadIdx.x; i < nl * ls; i += blockDim.x) A[i] = czero<T>();
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  // a warp takes up to kZGather rods at once and every lane issues all its
  // loads (up to 4 coefficients a rod) before it stores any: the gather is
  // latency bound, so the more loads in flight the better
  for (int rb = warp; rb < nl; rb += kZGather * nw) {
    RodInfo ri[kZGather];
    double2 v[kZGather][4];
#pragma unroll
    for (int r = 0; r < kZGather; ++r) {
      const int rl = rb + r * nw;
      ri[r] = rl < nl ? rods[r0 + rl] : RodInfo{0, 0, 0, 0};
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int i = lane + 32 * u;
        if (i < ri[r].size) v[r][u] = ps[ri[r].first + i];
      }
    }
#pragma unroll
    for (int r = 0; r < kZGather; ++r) {
      const int rl = rb + r * nw;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int i = lane + 32 * u;
        if (i < ri[r].size) {
          int z = ri[r].lmin + i;
          if (z < 0) z += n2;
          C c;
          c.x = from_f64<T>(v[r][u].x);
          c.y = from_f64<T>(v[r][u].y);
          A[rl * ls + z] = c;
        }
      }
      // rods longer than 128 coefficients
      for (int i = 128 + lane; i < ri[r].size; i += 32) {
        const double2 w = ps[ri[r].first + i];
        int z = ri[r].lmin + i;
        if (z < 0) z += n2;
        C c;
        c.x = from_f64<T>(w.x);
        c.y = from_f64<T>(w.y);
        A[rl * ls + z] = c;
      }
    }
  }
  __syncthreads();
  const C* R = A;
  if constexpr (L120) pfa120_inplace_lines<+1>(A, ls, nl);
  else R = fft_lines<+1, T, BIGP>(A, B, nl, ls, dv);
  C* Zs = Z + (size_t)blockIdx.y * n2 * nrods;
  const float inl = 1.f / (float)nl;
  for (int it = threadIdx.x; it < nl * n2; it += blockDim.x) {
    const int z = fdiv(it, inl), rl = it - z * nl;
    Zs[(size_t)z * nrods + r0 + rl] = R[rl * ls + z];
  }
}

// forward: read Z[s][z][rod], transform along z, scale by 1/N, scatter to
// the sphere with the epilogue of MODE:
//   0 store       c[g] = val
//   1 hpsi        o = (o_nl + kin*psi) + val; out[g] = o; acc[g] += fac*o
template <typename T, int MODE, bool BIGP, bool L120 = false>
__global__ void __launch_bounds__(kThreads)
k_z_fwd(const cplx<T>* __restrict__ Z, double2* out, int ldo,
        const RodInfo* __restrict__ rods, int nrods, FFTLen<T> d, T scale,
        const double2* psi, int ldp, const double* __restrict__ kpg2,
        int out_init, double2* acc, int lda, double2 fac) {
  // psi and acc may alias (the Taylor series is accumulated into the input
  // of the first H application); each element is read before it is written
  // by the same thread.
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem[];
  const int n2 = d.n, ls = n2 + 1;
  C* A = reinterpret_cast<C*>(smem);
  constexpr int TILE = L120 ? kTileZ120 : kTile;
  C* B = A + TILE * ls;
  const FFTLen<T> dv = stage_twiddles<T>(d, B + TILE * ls, BIGP);
  const int r0 = blockIdx.x * TILE;
  const int nl = min(TILE, nrods - r0);
  const int s = blockIdx.y;
  const C* Zs = Z + (size_t)s * n2 * nrods;
  {
    // eight loads in flight per thread before the stores (the Z rows come
    // from HBM and the load phase is latency bound)
    constexpr int U = 8;
    const int tot = nl * n2;
    const float inl = 1.f / (float)nl;
    for (int it0 = threadIdx.x; it0 < tot; it0 += U * blockDim.x) {
      C v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int it = it0 + u * blockDim.x;
        if (it < tot) {
          const int z = fdiv(it, inl), rl = it - z * nl;
          v[u] = Zs[(size_t)z * nrods + r0 + rl];
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int it = it0 + u * blockDim.x;
        if (it < tot) {
          const int z = fdiv(it, inl), rl = it - z * nl;
          A[rl * ls + z] = v[u];
        }
      }
    }
  }
  __syncthreads();
  const C* R = A;
  if constexpr (L120) pfa120_inplace_lines<-1>(A, ls, nl);
  else R = fft_lines<-1, T, BIGP>(A, B, nl, ls, dv);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  double2* os = out + (size_t)s * ldo;
  if constexpr (MODE == 2) {
    // scaled transform in the working type, in sphere order, for a separate
    // (coalesced) epilogue pass
    C* vs = reinterpret_cast<C*>(out) + (size_t)s * ldo;
    for (int rl = warp; rl < nl; rl += nw) {
      const RodInfo ri = rods[r0 + rl];
      for (int i = lane; i < ri.size; i += 32) {
        int z = ri.lmin + i;
        if (z < 0) z += n2;
        C vt = R[rl * ls + z];
        vt.x *= scale;
        vt.y *= scale;
        vs[ri.first + i] = vt;
      }
    }
    return;
  }
  if constexpr (std::is_same<T, df32>::value && MODE == 1) {
    // double-float arithmetic; FP64 only for the add of each stored
    // component.  A lane loads all its coefficients of a rod (up to four)
    // before computing, so the epilogue's loads overlap.
    constexpr int U = 4;
    const df32 fx = df32_from_f64(fac.x), fy = df32_from_f64(fac.y);
    for (int rl = warp; rl < nl; rl += nw) {
      const RodInfo ri = rods[r0 + rl];
      for (int ib = 0; ib < ri.size; ib += 32 * U) {
        double2 c64[U], o0[U], a0[U];
        double kp[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int i = ib + lane + 32 * u;
          if (i < ri.size) {
            const int g = ri.first + i;
            c64[u] = psi[(size_t)s * ldp + g];
            kp[u] = kpg2[g];
            o0[u] = out_init ? os[g] : make_double2(0.0, 0.0);
            if (acc) a0[u] = acc[(size_t)s * lda + g];
          }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int i = ib + lane + 32 * u;
          if (i < ri.size) {
            const int g = ri.first + i;
            int z = ri.lmin + i;
            if (z < 0) z += n2;
            C vt = R[rl * ls + z];
            const df32 xk = df_scale2(df32_from_f64(kp[u]), 0.5f);
            df32 ox = xk * df32_from_f64(c64[u].x), oy = xk * df32_from_f64(c64[u].y);
            if (out_init) {
              ox = ox + df32_from_f64(o0[u].x);
              oy = oy + df32_from_f64(o0[u].y);
            }
            ox = ox + vt.x * scale;
            oy = oy + vt.y * scale;
            os[g] = make_double2(f64_from_df32(ox), f64_from_df32(oy));
            if (acc) {
              const df32 ix = fx * ox - fy * oy, iy = fx * oy + fy * ox;
              acc[(size_t)s * lda + g] =
                  make_double2(a0[u].x + f64_from_df32(ix), a0[u].y + f64_from_df32(iy));
            }
          }
        }
      }
    }
    return;
  }
  for (int rl = warp; rl < nl; rl += nw) {
    const RodInfo ri = rods[r0 + rl];
    for (int i = lane; i < ri.size; i += 32) {
      int z = ri.lmin + i;
      if (z < 0) z += n2;
      C vt = R[rl * ls + z];
      vt.x *= scale;
      vt.y *= scale;
      const int g = ri.first + i;
      const double2 v = make_double2((double)vt.x, (double)vt.y);
      if (MODE == 0) {
        os[g] = v;
      } else {
        const double2 c = psi[(size_t)s * ldp + g];
        const double x = 0.5 * kpg2[g];
        double2 o = out_init ? os[g] : make_double2(0.0, 0.0);
        o.x = o.x + x * c.x;
        o.y = o.y + x * c.y;
        o.x = o.x + v.x;
        o.y = o.y + v.y;
        os[g] = o;
        if (acc) {
          double2* a = acc + (size_t)s * lda + g;
          const double ox = (double)o.x, oy = (double)o.y;
          double2 t = *a;
          t.x = t.x + (fac.x * ox - fac.y * oy);
          t.y = t.y + (fac.x * oy + fac.y * ox);
          *a = t;
        }
      }
    }
  }
}

// The H psi epilogue of the double-float form as its own pass over the
// sphere (coalesced, one thread per coefficient): out = (o_nl + kin c) + v,
// acc += fac out, with v the scaled forward transform stored by
// k_z_fwd<df32, 2>.  Double-float arithmetic; FP64 only for the add that
// forms each stored component.
__global__ void __launch_bounds__(256)
k_hpsi_epilogue_df32(const df32c* __restrict__ v, int ldv, const double2* psi, int ldp,
                     double2* out, int ldo, int out_init, const double* __restrict__ kpg2,
                     double2* acc, int lda, double2 fac, int ngw) {
  // psi and acc may alias: each element is read before it is written by the
  // same thread
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = blockIdx.y;
  if (g >= ngw) return;
  const double2 c64 = psi[(size_t)s * ldp + g];
  const double2 o0 = out_init ? out[(size_t)s * ldo + g] : make_double2(0.0, 0.0);
  const double2 a0 = acc ? acc[(size_t)s * lda + g] : make_double2(0.0, 0.0);
  const df32c vt = v[(size_t)s * ldv + g];
  const df32 xk = df_scale2(df32_from_f64(kpg2[g]), 0.5f);
  df32 ox = xk * df32_from_f64(c64.x), oy = xk * df32_from_f64(c64.y);
  if (out_init) {
    ox = ox + df32_from_f64(o0.x);
    oy = oy + df32_from_f64(o0.y);
  }
  ox = ox + vt.x;
  oy = oy + vt.y;
  out[(size_t)s * ldo + g] = make_double2(f64_from_df32(ox), f64_from_df32(oy));
  if (acc) {
    const df32 fx = df32_from_f64(fac.x), fy = df32_from_f64(fac.y);
    const df32 ix = fx * ox - fy * oy, iy = fx * oy + fy * ox;
    acc[(size_t)s * lda + g] = make_double2(a0.x + f64_from_df32(ix), a0.y + f64_from_df32(iy));
  }
}

// ------------------------------------------------------------------ x pass
template <typename T, bool BIGP>
__global__ void __launch_bounds__(kThreads)
k_x_bwd(const cplx<T>* __restrict__ Z, cplx<T>* __restrict__ Y, int nrods,
        int nband, int n2, const int* __restrict__ row_ptr,
        const int* __restrict__ row_rod, const int* __restrict__ row_xb,
        FFTLen<T> d) {
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem[];
  const int n0 = d.n, ls = n0 + 1;
  C* A = reinterpret_cast<C*>(smem);
  C* B = A + kTile * ls;
  const FFTLen<T> dv = stage_twiddles<T>(d, B + kTile * ls, BIGP);
  const int nbt = (nband + kTile - 1) / kTile;
  const int z = blockIdx.x / nbt;
  const int b0 = (blockIdx.x % nbt) * kTile;
  const int nl = min(kTile, nband - b0);
  const int s = blockIdx.y;
  for (int i = threadIdx.x; i < nl * ls; i += blockDim.x) A[i] = czero<T>();
  __syncthreads();
  const C* Zr = Z + ((size_t)s * n2 + z) * nrods;
  const int q1 = row_ptr[b0 + nl];
  for (int q = row_ptr[b0] + threadIdx.x; q < q1; q += blockDim.x) {
    const int xb = row_xb[q];
    A[((xb >> 16) - b0) * ls + (xb & 0xffff)] = Zr[row_rod[q]];
  }
  __syncthreads();
  const C* R = fft_lines<+1, T, BIGP>(A, B, nl, ls, dv);
  C* Yp = Y + ((size_t)s * n2 + z) * nband * n0;
  for (int it = threadIdx.x; it < nl * n0; it += blockDim.x) {
    const int bl = fdiv(it, 1.f / (float)n0), x = it - bl * n0;
    Yp[(size_t)(b0 + bl) * n0 + x] = R[bl * ls + x];
  }
}

template <typename T, bool BIGP>
__global__ void __launch_bounds__(kThreads)
k_x_fwd(const cplx<T>* __restrict__ Y, cplx<T>* __restrict__ Z, int nrods,
        int nband, int n2, const int* __restrict__ row_ptr,
        const int* __restrict__ row_rod, const int* __restrict__ row_xb,
        FFTLen<T> d) {
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem[];
  const int n0 = d.n, ls = n0 + 1;
  C* A = reinterpret_cast<C*>(smem);
  C* B = A + kTile * ls;
  const FFTLen<T> dv = stage_twiddles<T>(d, B + kTile * ls, BIGP);
  const int nbt = (nband + kTile - 1) / kTile;
  const int z = blockIdx.x / nbt;
  const int b0 = (blockIdx.x % nbt) * kTile;
  const int nl = min(kTile, nband - b0);
  const int s = blockIdx.y;
  const C* Yp = Y + ((size_t)s * n2 + z) * nband * n0;
  for (int it = threadIdx.x; it < nl * n0; it += blockDim.x) {
    const int bl = fdiv(it, 1.f / (float)n0), x = it - bl * n0;
    A[bl * ls + x] = Yp[(size_t)(b0 + bl) * n0 + x];
  }
  __syncthreads();
  const C* R = fft_lines<-1, T, BIGP>(A, B, nl, ls, dv);
  C* Zr = Z + ((size_t)s * n2 + z) * nrods;
  const int q1 = row_ptr[b0 + nl];
  for (int q = row_ptr[b0] + threadIdx.x; q < q1; q += blockDim.x) {
    const int xb = row_xb[q];
    Zr[row_rod[q]] = R[((xb >> 16) - b0) * ls + (xb & 0xffff)];
  }
}

// ------------------------------------------------------------------ y pass
enum YMode { Y_VLOC = 0, Y_BWD_STORE = 1, Y_FWD_LOAD = 2, Y_DENSITY = 3 };

template <typename T, int MODE, bool BIGP>
__global__ void __launch_bounds__(kThreads)
k_y(cplx<T>* __restrict__ Y, int nband, int n0, int n2,
    const int* __restrict__ band_y, const T* __restrict__ v,
    double2* __restrict__ f, const double* __restrict__ w, int nstates,
    double* __restrict__ rho, int rho_accumulate, FFTLen<T> d) {
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem[];
  const int n1 = d.n, ls = n1 + 1;
  C* A = reinterpret_cast<C*>(smem);
  C* B = A + kTile * ls;
  const FFTLen<T> dv = stage_twiddles<T>(d, B + kTile * ls, BIGP);
  const int nct = (n0 + kTile - 1) / kTile;
  const int z = blockIdx.x / nct;
  const int x0 = (blockIdx.x % nct) * kTile;
  const int nl = min(kTile, n0 - x0);
  const float inl = 1.f / (float)nl;
  const size_t plane = (size_t)n0 * n1;
  // v tile [n1][kTile], fetched asynchronously during the backward transform
  T* V = reinterpret_cast<T*>(A + fft_smem_elems(d, blockDim.x));
  if (MODE == Y_VLOC) {
    const T* vz = v + (size_t)z * plane;
    for (int it = threadIdx.x; it < nl * n1; it += blockDim.x) {
      const int y = fdiv(it, inl), cl = it - y * nl;
      cp_async<sizeof(T)>(V + y * kTile + cl, vz + (size_t)y * n0 + x0 + cl);
    }
    cp_async_commit();
  }
  {
    const int s = blockIdx.y;
    C* Yp = Y + ((size_t)s * n2 + z) * nband * n0;
    C* R;
    if (MODE == Y_FWD_LOAD) {
      const double2* fs = f + (size_t)s * plane * n2 + (size_t)z * plane;
      for (int it = threadIdx.x; it < nl * n1; it += blockDim.x) {
        const int y = fdiv(it, inl), cl = it - y * nl;
        const double2 fv = fs[(size_t)y * n0 + x0 + cl];
        C c;
        c.x = (T)fv.x;
        c.y = (T)fv.y;
        A[cl * ls + y] = c;
      }
      __syncthreads();
      R = fft_lines<-1, T, BIGP>(A, B, nl, ls, dv);
    } else {
      for (int i = threadIdx.x; i < nl * ls; i += blockDim.x) A[i] = czero<T>();
      __syncthreads();
      for (int it = threadIdx.x; it < nl * nband; it += blockDim.x) {
        const int b = fdiv(it, inl), cl = it - b * nl;
        A[cl * ls + band_y[b]] = Yp[(size_t)b * n0 + x0 + cl];
      }
      __syncthreads();
      R = fft_lines<+1, T, BIGP>(A, B, nl, ls, dv);
    }
    if (MODE == Y_VLOC) {
      // each thread reads back the v elements it fetched itself
      cp_async_wait_all();
      for (int it = threadIdx.x; it < nl * n1; it += blockDim.x) {
        const int y = fdiv(it, inl), cl = it - y * nl;
        const T vv = V[y * kTile + cl];
        C c = R[cl * ls + y];
        c.x = c.x * vv;
        c.y = c.y * vv;
        R[cl * ls + y] = c;
      }
      __syncthreads();
      C* other = R == A ? B : A;
      R = fft_lines<-1, T, BIGP>(R, other, nl, ls, dv);
    }
    if (MODE == Y_BWD_STORE) {
      double2* fs = f + (size_t)s * plane * n2 + (size_t)z * plane;
      for (int it = threadIdx.x; it < nl * n1; it += blockDim.x) {
        const int y = fdiv(it, inl), cl = it - y * nl;
        const C c = R[cl * ls + y];
        fs[(size_t)y * n0 + x0 + cl] = make_double2((double)c.x, (double)c.y);
      }
    } else if (MODE == Y_DENSITY) {
      // slot s of the density accumulates w_s |psi_s|^2 of this chunk's
      // state s; every slot element has exactly one writer per launch
      const double ws = w[s];
      double* rz = rho + (size_t)s * plane * n2 + (size_t)z * plane;
      for (int it = threadIdx.x; it < nl * n1; it += blockDim.x) {
        const int y = fdiv(it, inl), cl = it - y * nl;
        const C c = R[cl * ls + y];
        const double re = (double)c.x, im = (double)c.y;
        const double a = ws * (re * re + im * im);
        const size_t idx = (size_t)y * n0 + x0 + cl;
        rz[idx] = rho_accumulate ? rz[idx] + a : a;
      }
    } else {
      // VLOC, FWD_LOAD: keep the band rows
      for (int it = threadIdx.x; it < nl * nband; it += blockDim.x) {
        const int b = fdiv(it, inl), cl = it - b * nl;
        Yp[(size_t)b * n0 + x0 + cl] = R[cl * ls + band_y[b]];
      }
    }
  }
}

// rho[i] = sum_k slot[k][i] in slot order (deterministic): FP64 slots in
// FP64, double-float slots in double-float (the FP32 pipe; GB300 runs FP64
// at 1/72 of its rate) with one FP64 add for the stored value.  The loads
// of eight slots are issued before their adds.
template <typename ST> __device__ __forceinline__ double slot_f64(ST a) { return (double)a; }
template <> __device__ __forceinline__ double slot_f64<df32>(df32 a) { return f64_from_df32(a); }
template <typename ST>
__global__ void __launch_bounds__(256)
k_sum_slots(const ST* __restrict__ slots, int nslots, long long n, double* __restrict__ rho) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    ST a = slots[i];
    for (int k0 = 1; k0 < nslots; k0 += 8) {
      ST v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (k0 + u < nslots) v[u] = slots[(size_t)(k0 + u) * n + i];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (k0 + u < nslots) a = a + v[u];
    }
    rho[i] = slot_f64(a);
  }
}

// ---------------------------------------------- fused x -> y -> x pass
// The middle of one H psi transform for one (plane z, state s), all in
// shared memory: the plane's 2*ntrans0 band rows are filled from the z-pass
// output (one contiguous row of rods), transformed along x, then processed
// in groups of G columns -- zero-filled y lines, backward y transform,
// v(r) product (the v tile fetched with cp.async meanwhile), forward y
// transform, band rows written back -- and transformed forward along x;
// the rods go back to the same row of Z.  The Y intermediate of the
// three-kernel path never leaves the SM.  Needs prime-factor lengths along
// x and y that run in place, and the band rows plus one column group within
// one CTA's shared memory.
// the double-float H psi epilogue as a separate coalesced pass (1) or fused
// into the forward z pass (0)
#ifndef QBG_ZFWD_SPLIT
#define QBG_ZFWD_SPLIT 1
#endif
constexpr bool kZfwdSplit = QBG_ZFWD_SPLIT != 0;
#ifndef QBG_DENS_P3
#define QBG_DENS_P3 0
#endif
constexpr bool kDensP3 = QBG_DENS_P3 != 0;

// threads per CTA of the fused kernels: 768 for the three-pass 120-point
// transforms (their codelets fit 80 registers), 512 for the two-pass ones
#ifndef QBG_XYX_THREADS
#define QBG_XYX_THREADS 512
#endif
#ifndef QBG_XYX_THREADS_120
#define QBG_XYX_THREADS_120 768
#endif
template <int N> constexpr int xyx_threads() { return N == 120 ? QBG_XYX_THREADS_120 : QBG_XYX_THREADS; }

template <typename T, int X1, int X2, int Y1, int Y2>
__global__ void __launch_bounds__(xyx_threads<X1 * X2>(), 1)
k_xyx_vloc(cplx<T>* __restrict__ Z, int nrods, const int* __restrict__ row_rod,
           const int* __restrict__ row_xb, int nband, int n2, const T* __restrict__ v, int G) {
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int n0 = X1 * X2, n1 = Y1 * Y2, ls0 = n0 + 1, ls1 = n1 + 1;
  C* Xb = reinterpret_cast<C*>(smem);        // [nband][ls0]
  C* W = Xb + nband * ls0;                   // [G][ls1]
  T* V = reinterpret_cast<T*>(W + G * ls1);  // [n1][G]
  const int z = blockIdx.x, s = blockIdx.y;
  C* Zr = Z + ((size_t)s * n2 + z) * nrods;
  const size_t plane = (size_t)n0 * n1;
  for (int i = threadIdx.x; i < nband * ls0; i += blockDim.x) Xb[i] = czero<T>();
  __syncthreads();
  // band-row order: consecutive threads fill consecutive x of one row
  for (int q = threadIdx.x; q < nrods; q += blockDim.x) {
    const int xb = row_xb[q];
    Xb[(xb >> 16) * ls0 + (xb & 0xffff)] = Zr[row_rod[q]];
  }
  __syncthreads();
  constexpr bool kP3 = X1 * X2 == 120 && Y1 * Y2 == 120;  // three-pass 8 x 3 x 5
  constexpr int kThr = xyx_threads<X1 * X2>();
  constexpr int rg = kThr / X1;   // rows per in-place group (two passes)
  constexpr int rg3 = kThr / 15;  // rows per in-place group (three passes)
  if constexpr (kP3) {
    for (int b0 = 0; b0 < nband; b0 += rg3)
      pfa120_lines<+1>(Xb + b0 * ls0, ls0, min(rg3, nband - b0));
  } else {
    for (int b0 = 0; b0 < nband; b0 += rg)
      pfa_lines<X1, X2, +1, T>(Xb + b0 * ls0, nullptr, min(rg, nband - b0), ls0);
  }
  // y by column groups: fill, backward pass 1, backward pass 2 with the v
  // product fused into its stores, forward pass 1, forward pass 2 storing
  // only the band rows, straight into Xb
  using M = PfaMap<Y1, Y2>;
  const int nlow = nband / 2 + (nband & 1);  // band rows y < nlow are y = b
  const T* vz = v + (size_t)z * plane;
  for (int c0 = 0; c0 < n0; c0 += G) {
    const int gl = min(G, n0 - c0);
    const float igl = 1.f / (float)gl;
    for (int it = threadIdx.x; it < gl * n1; it += blockDim.x) {
      const int y = divf(it, igl), cl = it - y * gl;
      cp_async<sizeof(T)>(V + y * G + cl, vz + (size_t)y * n0 + c0 + cl);
    }
    cp_async_commit();
    for (int it = threadIdx.x; it < gl * n1; it += blockDim.x) {
      const int y = divf(it, igl), cl = it - y * gl;
      const int b = y < nlow ? y : (y >= n1 - (nband - nlow) ? y - n1 + nband : -1);
      W[cl * ls1 + y] = b >= 0 ? Xb[b * ls0 + c0 + cl] : czero<T>();
    }
    __syncthreads();
    if constexpr (kP3) {
      // 3- and 5-point passes, then the 8-point pass: backward with the v
      // product in its stores, forward storing only the band rows into Xb
      pfa120_ab<+1>(W, ls1, gl);
      const bool act3 = (int)threadIdx.x < gl * 15;
      const int j = divf(threadIdx.x, igl), cl3 = threadIdx.x - j * gl;
      const int ka = divf(j, 0.2f), kb = j - 5 * ka;
      C* ln3 = W + cl3 * ls1;
      C w8[8];
      if (act3) pfa120_c<+1>(ln3, ka, kb, w8);
      cp_async_wait_all();
      __syncthreads();
      if (act3) {
#pragma unroll
        for (int k1 = 0; k1 < 8; ++k1) {
          const int y = pfa120_out(k1, ka, kb);
          const T vv = V[y * G + cl3];
          C c = w8[k1];
          c.x = c.x * vv;
          c.y = c.y * vv;
          ln3[y] = c;
        }
      }
      __syncthreads();
      pfa120_ab<-1>(W, ls1, gl);
      if (act3) {
        pfa120_c<-1>(ln3, ka, kb, w8);
#pragma unroll
        for (int k1 = 0; k1 < 8; ++k1) {
          const int y = pfa120_out(k1, ka, kb);
          const int bb = y < nlow ? y : (y >= n1 - (nband - nlow) ? y - n1 + nband : -1);
          if (bb >= 0) Xb[bb * ls0 + c0 + cl3] = w8[k1];
        }
      }
      __syncthreads();
      continue;
    }
    for (int it = threadIdx.x; it < gl * Y2; it += blockDim.x) {
      const int n2i = it / gl;
      pfa_item1<Y1, Y2, +1>(W + (it - n2i * gl) * ls1, n2i);
    }
    cp_async_wait_all();
    __syncthreads();
    const bool act = (int)threadIdx.x < gl * Y1;
    const int k1 = threadIdx.x / gl;
    const int cl2 = threadIdx.x - k1 * gl;
    C* ln = W + cl2 * ls1;
    C u[Y2];
    if (act) {
#pragma unroll
      for (int b = 0; b < Y2; ++b) {
        int i2 = Y2 * k1 + Y1 * b;
        i2 = i2 >= M::N ? i2 - M::N : i2;
        u[b] = ln[i2];
      }
      dft_r<Y2, +1>(u, (const C*)nullptr, 0, 0, 0);
    }
    __syncthreads();
    if (act) {
      const int obase = (M::K1 * k1) % M::N;
#pragma unroll
      for (int b = 0; b < Y2; ++b) {
        int y = obase + (M::K2 * b) % M::N;
        y = y >= M::N ? y - M::N : y;
        const T vv = V[y * G + cl2];
        C c = u[b];
        c.x = c.x * vv;
        c.y = c.y * vv;
        ln[y] = c;
      }
    }
    __syncthreads();
    for (int it = threadIdx.x; it < gl * Y2; it += blockDim.x) {
      const int n2i = it / gl;
      pfa_item1<Y1, Y2, -1>(W + (it - n2i * gl) * ls1, n2i);
    }
    __syncthreads();
    if (act) {
#pragma unroll
      for (int b = 0; b < Y2; ++b) {
        int i2 = Y2 * k1 + Y1 * b;
        i2 = i2 >= M::N ? i2 - M::N : i2;
        u[b] = ln[i2];
      }
      dft_r<Y2, -1>(u, (const C*)nullptr, 0, 0, 0);
      const int obase = (M::K1 * k1) % M::N;
#pragma unroll
      for (int b = 0; b < Y2; ++b) {
        int y = obase + (M::K2 * b) % M::N;
        y = y >= M::N ? y - M::N : y;
        const int bb = y < nlow ? y : (y >= n1 - (nband - nlow) ? y - n1 + nband : -1);
        if (bb >= 0) Xb[bb * ls0 + c0 + cl2] = u[b];
      }
    }
    __syncthreads();
  }
  if constexpr (kP3) {
    for (int b0 = 0; b0 < nband; b0 += rg3)
      pfa120_lines<-1>(Xb + b0 * ls0, ls0, min(rg3, nband - b0));
  } else {
    for (int b0 = 0; b0 < nband; b0 += rg)
      pfa_lines<X1, X2, -1, T>(Xb + b0 * ls0, nullptr, min(rg, nband - b0), ls0);
  }
  for (int q = threadIdx.x; q < nrods; q += blockDim.x) {
    const int xb = row_xb[q];
    Zr[row_rod[q]] = Xb[(xb >> 16) * ls0 + (xb & 0xffff)];
  }
}

// Fused x -> y pass of the density for one (plane z, state s): band rows as
// in k_xyx_vloc, x backward, then per column group the backward y transform
// whose last pass writes w_s |psi(r)|^2 straight to density slot s.
// Density slots hold T-precision sums: double for FP64 transforms,
// double-float for double-float ones (|psi|^2 and the running sums then stay
// on the FP32 pipe; GB300 runs FP64 at 1/72 of the FP32 rate).
template <typename T> struct SlotOf { using type = double; };
template <> struct SlotOf<df32> { using type = df32; };

template <typename T, int X1, int X2, int Y1, int Y2>
__global__ void __launch_bounds__(xyx_threads<X1 * X2>(), 1)
k_xy_density(const cplx<T>* __restrict__ Z, int nrods, const int* __restrict__ row_rod,
             const int* __restrict__ row_xb, int nband, int n2, const double* __restrict__ w,
             typename SlotOf<T>::type* __restrict__ slots, int accumulate, int G) {
  using C = cplx<T>;
  using M = PfaMap<Y1, Y2>;
  using ST = typename SlotOf<T>::type;
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int n0 = X1 * X2, n1 = Y1 * Y2, ls0 = n0 + 1, ls1 = n1 + 1;
  C* Xb = reinterpret_cast<C*>(smem);  // [nband][ls0]
  C* W = Xb + nband * ls0;             // [G][ls1]
  const int z = blockIdx.x, s = blockIdx.y;
  const C* Zr = Z + ((size_t)s * n2 + z) * nrods;
  const size_t plane = (size_t)n0 * n1;
  ST* rz = slots + (size_t)s * plane * n2 + (size_t)z * plane;
  const T ws = T(w[s]);
  for (int i = threadIdx.x; i < nband * ls0; i += blockDim.x) Xb[i] = czero<T>();
  __syncthreads();
  // band-row order: consecutive threads fill consecutive x of one row
  for (int q = threadIdx.x; q < nrods; q += blockDim.x) {
    const int xb = row_xb[q];
    Xb[(xb >> 16) * ls0 + (xb & 0xffff)] = Zr[row_rod[q]];
  }
  __syncthreads();
  constexpr bool kP3 = X1 * X2 == 120 && Y1 * Y2 == 120;
  constexpr int kThr = xyx_threads<X1 * X2>();
  constexpr int rg = kThr / X1;
  constexpr int rg3 = kThr / 15;
  if constexpr (kP3) {
    for (int b0 = 0; b0 < nband; b0 += rg3)
      pfa120_lines<+1>(Xb + b0 * ls0, ls0, min(rg3, nband - b0));
  } else {
    for (int b0 = 0; b0 < nband; b0 += rg)
      pfa_lines<X1, X2, +1, T>(Xb + b0 * ls0, nullptr, min(rg, nband - b0), ls0);
  }
  // column groups; when accumulating, the slot tile of the group is fetched
  // with cp.async into S while the group is filled and transformed
  ST* S = reinterpret_cast<ST*>(W + G * ls1);  // [n1][G]
  const int nlow = nband / 2 + (nband & 1);
  for (int c0 = 0; c0 < n0; c0 += G) {
    const int gl = min(G, n0 - c0);
    const float igl = 1.f / (float)gl;
    if (accumulate) {
      for (int it = threadIdx.x; it < gl * n1; it += blockDim.x) {
        const int y = divf(it, igl), cl = it - y * gl;
        cp_async<sizeof(ST)>(S + y * G + cl, rz + (size_t)y * n0 + c0 + cl);
      }
      cp_async_commit();
    }
    for (int it = threadIdx.x; it < gl * n1; it += blockDim.x) {
      const int y = divf(it, igl), cl = it - y * gl;
      const int b = y < nlow ? y : (y >= n1 - (nband - nlow) ? y - n1 + nband : -1);
      W[cl * ls1 + y] = b >= 0 ? Xb[b * ls0 + c0 + cl] : czero<T>();
    }
    __syncthreads();
    // (the y pass keeps the two-pass split by default: with no forward
    // half, its last pass writes straight to memory)
    if constexpr (kP3 && kDensP3) {
      pfa120_ab<+1>(W, ls1, gl);
      if (accumulate) {
        cp_async_wait_all();
        __syncthreads();
      }
      if ((int)threadIdx.x < gl * 15) {
        const int j = divf(threadIdx.x, igl), cl3 = threadIdx.x - j * gl;
        const int ka = divf(j, 0.2f), kb = j - 5 * ka;
        C w8[8];
        pfa120_c<+1>(W + cl3 * ls1, ka, kb, w8);
#pragma unroll
        for (int k1 = 0; k1 < 8; ++k1) {
          const int y = pfa120_out(k1, ka, kb);
          const T a = ws * (w8[k1].x * w8[k1].x + w8[k1].y * w8[k1].y);
          rz[(size_t)y * n0 + c0 + cl3] = accumulate ? S[y * G + cl3] + a : a;
        }
      }
      __syncthreads();
      continue;
    }
    for (int it = threadIdx.x; it < gl * Y2; it += blockDim.x) {
      const int n2i = it / gl;
      pfa_item1<Y1, Y2, +1>(W + (it - n2i * gl) * ls1, n2i);
    }
    if (accumulate) cp_async_wait_all();
    __syncthreads();
    if ((int)threadIdx.x < gl * Y1) {
      const int k1 = threadIdx.x / gl;
      const int cl2 = threadIdx.x - k1 * gl;
      const C* ln = W + cl2 * ls1;
      C u[Y2];
#pragma unroll
      for (int b = 0; b < Y2; ++b) {
        int i2 = Y2 * k1 + Y1 * b;
        i2 = i2 >= M::N ? i2 - M::N : i2;
        u[b] = ln[i2];
      }
      dft_r<Y2, +1>(u, (const C*)nullptr, 0, 0, 0);
      const int obase = (M::K1 * k1) % M::N;
#pragma unroll
      for (int b = 0; b < Y2; ++b) {
        int y = obase + (M::K2 * b) % M::N;
        y = y >= M::N ? y - M::N : y;
        const T a = ws * (u[b].x * u[b].x + u[b].y * u[b].y);
        rz[(size_t)y * n0 + c0 + cl2] = accumulate ? S[y * G + cl2] + a : a;
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------- lane-group y pass
// The y pass of the local-potential product with register-resident columns:
// each group of B lanes owns one column x of a plane (n1 = A*B values), does
// the backward transform (L1 -> L2), multiplies by v(x, y, z) in the L2
// layout and transforms forward (L2 -> L1) with no shared-memory round trip
// or barrier in between.  Shared memory only stages the band-row tile and
// the v tile so that global accesses stay coalesced.
constexpr int kLgThreads = 128;

template <typename T, int A, int B>
__global__ void __launch_bounds__(kLgThreads)
k_y_lg_vloc(cplx<T>* __restrict__ Y, int nband, int ntrans0, int n0, int n2,
            const T* __restrict__ v, FFTLen<T> d) {
  using C = cplx<T>;
  constexpr int n1 = A * B;
  constexpr int CPC = (kLgThreads / 32) * (32 / B);  // columns per CTA
  constexpr int LD = CPC + 1;
  extern __shared__ __align__(16) unsigned char smem[];
  C* Wn = reinterpret_cast<C*>(smem);                 // n1 roots
  C* T_ = Wn + n1;                                    // [nband][LD]
  T* V = reinterpret_cast<T*>(T_ + (size_t)nband * LD);  // [n1][LD]
  const int nct = (n0 + CPC - 1) / CPC;
  const int z = blockIdx.x / nct;
  const int x0 = (blockIdx.x % nct) * CPC;
  const int s = blockIdx.y;
  const int ncol = min(CPC, n0 - x0);
  C* Yp = Y + ((size_t)s * n2 + z) * nband * n0;
  const T* vz = v + (size_t)z * n0 * n1;
  for (int i = threadIdx.x; i < n1; i += blockDim.x) Wn[i] = d.root[i];
  for (int it = threadIdx.x; it < nband * CPC; it += blockDim.x) {
    const int b = it / CPC, c = it - b * CPC;
    if (c < ncol) T_[b * LD + c] = Yp[(size_t)b * n0 + x0 + c];
  }
  for (int it = threadIdx.x; it < n1 * CPC; it += blockDim.x) {
    const int y = it / CPC, c = it - y * CPC;
    if (c < ncol) V[y * LD + c] = vz[(size_t)y * n0 + x0 + c];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int b = lane & (B - 1);
  const int c = (threadIdx.x >> 5) * (32 / B) + lane / B;
  const bool live = c < ncol;
  C r[A];
#pragma unroll
  for (int a = 0; a < A; ++a) {
    const int y = b + B * a;
    const int bi = y < ntrans0 ? y : (y >= n1 - ntrans0 ? y - n1 + nband : -1);
    r[a] = (live && bi >= 0) ? T_[bi * LD + c] : cmk<C>(T(0), T(0));
  }
  regs_then_lanes<+1, A, B>(r, b, Wn);
  const int rb = lane_rev<B>(b);
#pragma unroll
  for (int a = 0; a < A; ++a) {
    const T vv = live ? V[(a + A * rb) * LD + c] : T(0);
    r[a].x = r[a].x * vv;
    r[a].y = r[a].y * vv;
  }
  lanes_then_regs<-1, A, B>(r, b, Wn);
  __syncthreads();
#pragma unroll
  for (int a = 0; a < A; ++a) {
    const int y = b + B * a;
    const int bi = y < ntrans0 ? y : (y >= n1 - ntrans0 ? y - n1 + nband : -1);
    if (live && bi >= 0) T_[bi * LD + c] = r[a];
  }
  __syncthreads();
  for (int it = threadIdx.x; it < nband * CPC; it += blockDim.x) {
    const int bb = it / CPC, cc = it - bb * CPC;
    if (cc < ncol) Yp[(size_t)bb * n0 + x0 + cc] = T_[bb * LD + cc];
  }
}

// ------------------------------------------------------------- launchers
// threads per CTA: the prime-factor passes of a 16-line tile have 15 and 8
// items per line (120 = 8 x 15), so 128 threads keep both passes busy and
// leave room for more resident CTAs; the Stockham passes use 256
#ifndef QBG_PFA_THREADS
#define QBG_PFA_THREADS 128
#endif
#ifndef QBG_PFA_THREADS_Z
#define QBG_PFA_THREADS_Z 128
#endif
template <typename T> static int nthreads(const FFTLen<T>& d) {
  return d.pfa ? QBG_PFA_THREADS : kThreads;
}
// z passes: the sphere gather/scatter epilogue runs one warp per rod
template <typename T> static int nthreads_z(const FFTLen<T>& d) {
  return d.pfa ? QBG_PFA_THREADS_Z : kThreads;
}

template <typename T> static size_t smem_bytes(const FFTLen<T>& d, bool vtile = false,
                                               int threads = 0) {
  return (size_t)fft_smem_elems(d, threads ? threads : nthreads(d)) * sizeof(cplx<T>) +
         (vtile ? (size_t)d.n * kTile * sizeof(T) : 0);
}

template <typename K> static cudaError_t prep(K kernel, size_t smem) {
  if (smem > 48 * 1024)
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return cudaSuccess;
}

template <typename T> static qbg_status ensure_scratch(qbg_plan* p, int nch) {
  const size_t zb = (size_t)nch * p->np2 * p->nrods * sizeof(cplx<T>);
  const size_t yb = (size_t)nch * p->np2 * p->nband * p->np0 * sizeof(cplx<T>);
  qbg_status s = ensure(&p->d_Z, &p->Z_bytes, zb);
  if (s) return s;
  return ensure(&p->d_Y, &p->Y_bytes, yb);
}

static bool big_prime(const LenTables& L) {
  for (int i = 0; i < L.npass; ++i)
    if (L.radix[i] == 7 || L.radix[i] == 11 || L.radix[i] == 13) return true;
  return false;
}

// The launchers below work on the plan's Z and Y intermediates unless the
// caller passes its own (Z, Y: the same shapes for ns states).
// z lines of 120 points as the in-place three-pass prime-factor transform
// (with the whole-plane kernels: the plan's fused mode 2)
template <typename T> static bool z_inplace120(const qbg_plan* p, const FFTLen<T>& d) {
  return d.n == 120 && d.pfa && p->fuse_xyx && p->plane_xyx;
}

template <typename T, bool BIGP>
static qbg_status run_z_bwd_(qbg_plan* p, const double2* c, int ldc, int ns, cudaStream_t st,
                             void* Z) {
  const FFTLen<T> d = p->len[2].view<T>();
  const size_t sm = smem_bytes<T>(d, false, nthreads_z(d));
  dim3 grid((p->nrods + kTile - 1) / kTile, ns);
  PhaseTimer pt(p, PH_Z_BWD, st);
  if (!BIGP && z_inplace120(p, d)) {
    QBG_CUDA(prep(k_z_bwd<T, false, true>, sm));
    k_z_bwd<T, false, true><<<grid, nthreads_z(d), sm, st>>>(
        c, ldc, (cplx<T>*)(Z ? Z : p->d_Z), p->d_rods, p->nrods, d);
  } else {
    QBG_CUDA(prep(k_z_bwd<T, BIGP>, sm));
    k_z_bwd<T, BIGP><<<grid, nthreads_z(d), sm, st>>>(c, ldc, (cplx<T>*)(Z ? Z : p->d_Z),
                                                      p->d_rods, p->nrods, d);
  }
  QBG_LAUNCHED(p);
  return QBG_OK;
}
template <typename T>
static qbg_status run_z_bwd(qbg_plan* p, const double2* c, int ldc, int ns, cudaStream_t st,
                            void* Z = nullptr) {
  return big_prime(p->len[2]) ? run_z_bwd_<T, true>(p, c, ldc, ns, st, Z)
                              : run_z_bwd_<T, false>(p, c, ldc, ns, st, Z);
}

template <typename T, bool BIGP>
static qbg_status run_x_(qbg_plan* p, bool bwd, int ns, cudaStream_t st, void* Z, void* Y) {
  const FFTLen<T> d = p->len[0].view<T>();
  const size_t sm = smem_bytes<T>(d);
  dim3 grid(p->np2 * ((p->nband + kTile - 1) / kTile), ns);
  cplx<T>* z = (cplx<T>*)(Z ? Z : p->d_Z);
  cplx<T>* y = (cplx<T>*)(Y ? Y : p->d_Y);
  PhaseTimer pt(p, bwd ? PH_X_BWD : PH_X_FWD, st);
  if (bwd) {
    QBG_CUDA(prep(k_x_bwd<T, BIGP>, sm));
    k_x_bwd<T, BIGP><<<grid, nthreads(d), sm, st>>>(z, y, p->nrods, p->nband, p->np2,
                                                    p->d_row_ptr, p->d_row_rod, p->d_row_x, d);
  } else {
    QBG_CUDA(prep(k_x_fwd<T, BIGP>, sm));
    k_x_fwd<T, BIGP><<<grid, nthreads(d), sm, st>>>(y, z, p->nrods, p->nband, p->np2,
                                                    p->d_row_ptr, p->d_row_rod, p->d_row_x, d);
  }
  QBG_LAUNCHED(p);
  return QBG_OK;
}
template <typename T>
static qbg_status run_x(qbg_plan* p, bool bwd, int ns, cudaStream_t st, void* Z = nullptr,
                        void* Y = nullptr) {
  return big_prime(p->len[0]) ? run_x_<T, true>(p, bwd, ns, st, Z, Y)
                              : run_x_<T, false>(p, bwd, ns, st, Z, Y);
}

template <typename T, int MODE, bool BIGP>
static qbg_status run_y_(qbg_plan* p, int ns, double2* f, const double* w, double* rho,
                         int rho_acc, cudaStream_t st, void* Y = nullptr) {
  const FFTLen<T> d = p->len[1].view<T>();
  const size_t sm = smem_bytes<T>(d, MODE == Y_VLOC);
  QBG_CUDA(prep(k_y<T, MODE, BIGP>, sm));
  dim3 grid(p->np2 * ((p->np0 + kTile - 1) / kTile), ns);
  PhaseTimer pt(p, MODE == Y_VLOC ? PH_Y_VLOC : MODE == Y_DENSITY ? PH_Y_DENSITY
                   : MODE == Y_BWD_STORE ? PH_Y_STORE : PH_Y_LOAD, st);
  const T* v = nullptr;
  if (MODE == Y_VLOC)
    v = std::is_same<T, double>::value  ? (const T*)p->d_vr
        : std::is_same<T, float>::value ? (const T*)p->d_vr32
                                        : (const T*)p->d_vrdf;
  k_y<T, MODE, BIGP><<<grid, nthreads(d), sm, st>>>((cplx<T>*)(Y ? Y : p->d_Y), p->nband,
                                                    p->np0, p->np2, p->d_band_y, v, f, w, ns,
                                                    rho, rho_acc, d);
  QBG_LAUNCHED(p);
  return QBG_OK;
}
template <typename T, int A, int B>
static qbg_status run_y_lg_vloc(qbg_plan* p, int ns, cudaStream_t st) {
  const FFTLen<T> d = p->len[1].view<T>();
  constexpr int CPC = (kLgThreads / 32) * (32 / B);
  const size_t sm = (size_t)A * B * sizeof(cplx<T>) + (size_t)p->nband * (CPC + 1) * sizeof(cplx<T>) +
                    (size_t)A * B * (CPC + 1) * sizeof(T);
  QBG_CUDA(prep(k_y_lg_vloc<T, A, B>, sm));
  const T* v = std::is_same<T, double>::value  ? (const T*)p->d_vr
               : std::is_same<T, float>::value ? (const T*)p->d_vr32
                                               : (const T*)p->d_vrdf;
  dim3 grid(p->np2 * ((p->np0 + CPC - 1) / CPC), ns);
  PhaseTimer pt(p, PH_Y_VLOC, st);
  k_y_lg_vloc<T, A, B><<<grid, kLgThreads, sm, st>>>((cplx<T>*)p->d_Y, p->nband, p->ntrans0,
                                                     p->np0, p->np2, v, d);
  QBG_LAUNCHED(p);
  return QBG_OK;
}

// lane-group split of the y length, or 0 when the Stockham engine is used
static int lg_split(int n1) {
  switch (n1) {
    case 32: return 4 * 100 + 8;
    case 48: return 6 * 100 + 8;
    case 64: return 8 * 100 + 8;
    case 96: return 12 * 100 + 8;
    case 120: return 15 * 100 + 8;
    case 144: return 9 * 100 + 16;
    case 160: return 10 * 100 + 16;
    default: return 0;
  }
}

template <typename T>
static qbg_status run_y_vloc(qbg_plan* p, int ns, cudaStream_t st, bool* done) {
  *done = true;
  // the shuffle network's per-stage twiddles pay off only where the pass is
  // latency bound (FP32); the FP64 and double-float passes are arithmetic
  // bound and run faster through the shared-memory radix-8/3/5 engine
  if (!p->lane_fft || !std::is_same<T, float>::value) {
    *done = false;
    return QBG_OK;
  }
  switch (lg_split(p->np1)) {
    case 408: return run_y_lg_vloc<T, 4, 8>(p, ns, st);
    case 608: return run_y_lg_vloc<T, 6, 8>(p, ns, st);
    case 808: return run_y_lg_vloc<T, 8, 8>(p, ns, st);
    case 1208: return run_y_lg_vloc<T, 12, 8>(p, ns, st);
    case 1508: return run_y_lg_vloc<T, 15, 8>(p, ns, st);
    case 916: return run_y_lg_vloc<T, 9, 16>(p, ns, st);
    case 1016: return run_y_lg_vloc<T, 10, 16>(p, ns, st);
    default: *done = false; return QBG_OK;
  }
}

template <typename T, int MODE>
static qbg_status run_y(qbg_plan* p, int ns, double2* f, const double* w, double* rho,
                        int rho_acc, cudaStream_t st) {
  if (MODE == Y_VLOC) {
    bool done = false;
    qbg_status s = run_y_vloc<T>(p, ns, st, &done);
    if (done || s != QBG_OK) return s;
  }
  return big_prime(p->len[1]) ? run_y_<T, MODE, true>(p, ns, f, w, rho, rho_acc, st)
                              : run_y_<T, MODE, false>(p, ns, f, w, rho, rho_acc, st);
}

template <typename T, int MODE, bool BIGP>
static qbg_status run_z_fwd_(qbg_plan* p, double2* out, int ldo, int ns, const double2* psi,
                             int ldp, int out_init, double2* acc, int lda, double2 fac,
                             cudaStream_t st) {
  const FFTLen<T> d = p->len[2].view<T>();
  const size_t sm = smem_bytes<T>(d, false, nthreads_z(d));
  dim3 grid((p->nrods + kTile - 1) / kTile, ns);
  const T scale = (T)(1.0 / (double)(p->np0 * p->np1 * p->np2));
  const double* kin = p->d_kpg2A;
  PhaseTimer pt(p, PH_Z_FWD, st);
  if (!BIGP && z_inplace120(p, d)) {
    const size_t sm120 = sizeof(cplx<T>) * (size_t)kTileZ120 * (d.n + 1);
    const dim3 grid120((p->nrods + kTileZ120 - 1) / kTileZ120, ns);
    QBG_CUDA(prep(k_z_fwd<T, MODE, false, true>, sm120));
    k_z_fwd<T, MODE, false, true><<<grid120, kThreads, sm120, st>>>(
        (const cplx<T>*)p->d_Z, out, ldo, p->d_rods, p->nrods, d, scale, psi, ldp, kin,
        out_init, acc, lda, fac);
  } else {
    QBG_CUDA(prep(k_z_fwd<T, MODE, BIGP>, sm));
    k_z_fwd<T, MODE, BIGP><<<grid, nthreads_z(d), sm, st>>>((const cplx<T>*)p->d_Z, out, ldo,
                                                      p->d_rods, p->nrods, d, scale, psi, ldp,
                                                      kin, out_init, acc, lda, fac);
  }
  QBG_LAUNCHED(p);
  return QBG_OK;
}
template <typename T, int MODE>
static qbg_status run_z_fwd(qbg_plan* p, double2* out, int ldo, int ns, const double2* psi,
                            int ldp, int out_init, double2* acc, int lda, double2 fac,
                            cudaStream_t st) {
  return big_prime(p->len[2])
             ? run_z_fwd_<T, MODE, true>(p, out, ldo, ns, psi, ldp, out_init, acc, lda, fac, st)
             : run_z_fwd_<T, MODE, false>(p, out, ldo, ns, psi, ldp, out_init, acc, lda, fac, st);
}

#define QBG_TRY(x)                \
  do {                            \
    qbg_status s_ = (x);          \
    if (s_ != QBG_OK) return s_;  \
  } while (0)

template <typename T, int X1, int X2, int Y1, int Y2>
static qbg_status run_xyx_(qbg_plan* p, int ns, int G, size_t sm, cudaStream_t st) {
  QBG_CUDA(prep(k_xyx_vloc<T, X1, X2, Y1, Y2>, sm));
  const T* v = std::is_same<T, double>::value ? (const T*)p->d_vr : (const T*)p->d_vrdf;
  PhaseTimer pt(p, PH_XYX_VLOC, st);
  k_xyx_vloc<T, X1, X2, Y1, Y2><<<dim3(p->np2, ns), xyx_threads<X1 * X2>(), sm, st>>>(
      (cplx<T>*)p->d_Z, p->nrods, p->d_row_rod, p->d_row_x, p->nband, p->np2, v, G);
  QBG_LAUNCHED(p);
  return QBG_OK;
}
// (n0, n1) pairs with a compiled fused kernel
static bool xyx_lengths(int n0, int n1) {
  return n0 == n1 && (n0 == 120 || n0 == 48 || n0 == 40);
}
template <typename T, int X1, int X2, int Y1, int Y2>
static qbg_status run_xy_density_(qbg_plan* p, int ns, const double* w, int acc, int G,
                                  size_t sm, cudaStream_t st) {
  QBG_CUDA(prep(k_xy_density<T, X1, X2, Y1, Y2>, sm));
  PhaseTimer pt(p, PH_Y_DENSITY, st);
  k_xy_density<T, X1, X2, Y1, Y2><<<dim3(p->np2, ns), xyx_threads<X1 * X2>(), sm, st>>>(
      (const cplx<T>*)p->d_Z, p->nrods, p->d_row_rod, p->d_row_x, p->nband, p->np2, w,
      (typename SlotOf<T>::type*)p->d_rho_slots, acc, G);
  QBG_LAUNCHED(p);
  return QBG_OK;
}
template <typename T>
static qbg_status run_xy_density(qbg_plan* p, int ns, const double* w, int acc, int G,
                                 size_t sm, cudaStream_t st) {
  switch (p->np0) {
    case 120: return run_xy_density_<T, 8, 15, 8, 15>(p, ns, w, acc, G, sm, st);
    case 48: return run_xy_density_<T, 16, 3, 16, 3>(p, ns, w, acc, G, sm, st);
    default: return run_xy_density_<T, 8, 5, 8, 5>(p, ns, w, acc, G, sm, st);
  }
}

template <typename T>
static qbg_status run_xyx(qbg_plan* p, int ns, int G, size_t sm, cudaStream_t st) {
  switch (p->np0) {
    case 120: return run_xyx_<T, 8, 15, 8, 15>(p, ns, G, sm, st);
    case 48: return run_xyx_<T, 16, 3, 16, 3>(p, ns, G, sm, st);
    default: return run_xyx_<T, 8, 5, 8, 5>(p, ns, G, sm, st);
  }
}

// Column-group width of the fused x -> y -> x kernel, 0 when it does not
// apply (lengths without an in-place prime-factor split, or shared memory).
template <typename T> static int xyx_group(const qbg_plan* p, size_t* smem) {
  const FFTLen<T> dx = p->len[0].view<T>(), dy = p->len[1].view<T>();
  if (!p->fuse_xyx || !xyx_lengths(p->np0, p->np1) || std::is_same<T, float>::value) return 0;
  if (!dx.pfa || !dy.pfa) return 0;  // the fused kernel runs prime-factor splits in place
  const size_t cs = sizeof(cplx<T>);
  const size_t base = (size_t)p->nband * (p->np0 + 1) * cs;
  const size_t per_col = (size_t)(p->np1 + 1) * cs + (size_t)p->np1 * sizeof(T);
  const size_t cap = 227 * 1024;
  const int thr = p->np0 == 120 ? xyx_threads<120>() : xyx_threads<0>();
  if (base + per_col > cap || thr / dx.pfa < 1) return 0;
  const int gmax = std::min<int>({(int)((cap - base) / per_col), thr / dy.pfa, p->np0});
  if (gmax < 8) return 0;
  const int ngroups = (p->np0 + gmax - 1) / gmax;
  const int G = (p->np0 + ngroups - 1) / ngroups;
  *smem = base + (size_t)G * per_col;
  return G;
}

// Column-group width of the fused density kernel (0: not applicable).
template <typename T> static int xy_density_group(const qbg_plan* p, size_t* smem) {
  if (!p->fuse_xyx || !xyx_lengths(p->np0, p->np1) || std::is_same<T, float>::value) return 0;
  const FFTLen<T> dy = p->len[1].view<T>();
  if (!dy.pfa || !p->len[0].view<T>().pfa) return 0;
  const size_t cs = sizeof(cplx<T>);
  const size_t base = (size_t)p->nband * (p->np0 + 1) * cs;
  const size_t per_col = (size_t)(p->np1 + 1) * cs + (size_t)p->np1 * sizeof(double);
  const size_t cap = 227 * 1024;
  if (base + per_col > cap) return 0;
  const int thr = p->np0 == 120 ? xyx_threads<120>() : xyx_threads<0>();
  const int gmax = std::min<int>({(int)((cap - base) / per_col), thr / dy.pfa, p->np0});
  if (gmax < 8) return 0;
  const int ngroups = (p->np0 + gmax - 1) / gmax;
  const int G = (p->np0 + ngroups - 1) / ngroups;
  *smem = base + (size_t)G * per_col;
  return G;
}

template <typename T>
qbg_status local_hpsi(qbg_plan* p, const double2* psi, int ld, double2* out, int nst,
                      bool out_init, double2* acc, int ldacc, double2 fac, cudaStream_t st) {
  const int ch = std::max(1, std::min(p->chunk, nst));
  QBG_TRY(ensure_scratch<T>(p, ch));
  size_t xyx_smem = 0;
  const bool plane = plane_applies(p, std::is_same<T, float>::value);
  const int G = plane ? 0 : xyx_group<T>(p, &xyx_smem);
  for (int s0 = 0; s0 < nst; s0 += ch) {
    const int ns = std::min(ch, nst - s0);
    QBG_TRY(run_z_bwd<T>(p, psi + (size_t)s0 * ld, ld, ns, st));
    if (plane) {
      if constexpr (!std::is_same<T, float>::value) QBG_TRY(plane_vloc<T>(p, ns, s0, st));
    } else if (G) {
      if constexpr (!std::is_same<T, float>::value) QBG_TRY(run_xyx<T>(p, ns, G, xyx_smem, st));
    } else {
      QBG_TRY(run_x<T>(p, true, ns, st));
      QBG_TRY((run_y<T, Y_VLOC>(p, ns, nullptr, nullptr, nullptr, 0, st)));
      QBG_TRY(run_x<T>(p, false, ns, st));
    }
    if (std::is_same<T, df32>::value && kZfwdSplit) {
      QBG_TRY(ensure(&p->d_vsph, &p->vsph_bytes, sizeof(df32c) * (size_t)ch * p->ngw));
      QBG_TRY((run_z_fwd<T, 2>(p, (double2*)p->d_vsph, p->ngw, ns, nullptr, 0, 0, nullptr, 0,
                               fac, st)));
      PhaseTimer pt(p, PH_Z_FWD, st);
      k_hpsi_epilogue_df32<<<dim3((p->ngw + 255) / 256, ns), 256, 0, st>>>(
          (const df32c*)p->d_vsph, p->ngw, psi + (size_t)s0 * ld, ld, out + (size_t)s0 * ld, ld,
          out_init ? 1 : 0, p->d_kpg2A, acc ? acc + (size_t)s0 * ldacc : nullptr, ldacc, fac,
          p->ngw);
      QBG_LAUNCHED(p);
    } else {
      QBG_TRY((run_z_fwd<T, 1>(p, out + (size_t)s0 * ld, ld, ns, psi + (size_t)s0 * ld, ld,
                               out_init ? 1 : 0, acc ? acc + (size_t)s0 * ldacc : nullptr, ldacc,
                               fac, st)));
    }
  }
  return QBG_OK;
}

template <typename T>
qbg_status backward(qbg_plan* p, const double2* c, int ldc, double2* f, int nb, cudaStream_t st) {
  const int ch = std::max(1, std::min(p->chunk, nb));
  QBG_TRY(ensure_scratch<T>(p, ch));
  for (int s0 = 0; s0 < nb; s0 += ch) {
    const int ns = std::min(ch, nb - s0);
    QBG_TRY(run_z_bwd<T>(p, c + (size_t)s0 * ldc, ldc, ns, st));
    if (plane_applies(p, std::is_same<T, float>::value)) {
      if constexpr (!std::is_same<T, float>::value)
        QBG_TRY(plane_field<T>(p, ns, f + (size_t)s0 * p->N, st));
      continue;
    }
    QBG_TRY(run_x<T>(p, true, ns, st));
    QBG_TRY((run_y<T, Y_BWD_STORE>(p, ns, f + (size_t)s0 * p->N, nullptr, nullptr, 0, st)));
  }
  return QBG_OK;
}

template <typename T>
qbg_status plane_fields(qbg_plan* p, const double2* c, int ld, int nst, void* F,
                        cudaStream_t st) {
  if constexpr (std::is_same<T, float>::value) {
    set_error("plane_fields: no whole-plane kernel for FP32 transforms");
    return QBG_ERR_UNSUPPORTED;
  } else {
    const int ch = std::max(1, std::min(p->chunk, nst));
    QBG_TRY(ensure_scratch<T>(p, ch));
    for (int s0 = 0; s0 < nst; s0 += ch) {
      const int ns = std::min(ch, nst - s0);
      QBG_TRY(run_z_bwd<T>(p, c + (size_t)s0 * ld, ld, ns, st));
      QBG_TRY(plane_pair_field<T>(p, ns, (cplx<T>*)F + (size_t)s0 * p->N, st));
    }
    return QBG_OK;
  }
}
template qbg_status plane_fields<double>(qbg_plan*, const double2*, int, int, void*,
                                         cudaStream_t);
template qbg_status plane_fields<df32>(qbg_plan*, const double2*, int, int, void*, cudaStream_t);

template <typename T>
qbg_status forward(qbg_plan* p, double2* f, double2* c, int ldc, int nb, cudaStream_t st) {
  const int ch = std::max(1, std::min(p->chunk, nb));
  QBG_TRY(ensure_scratch<T>(p, ch));
  const double2 zero = make_double2(0.0, 0.0);
  for (int s0 = 0; s0 < nb; s0 += ch) {
    const int ns = std::min(ch, nb - s0);
    if (plane_applies(p, std::is_same<T, float>::value)) {
      if constexpr (!std::is_same<T, float>::value)
        QBG_TRY(plane_fwd<T>(p, ns, f + (size_t)s0 * p->N, st));
    } else {
      QBG_TRY((run_y<T, Y_FWD_LOAD>(p, ns, f + (size_t)s0 * p->N, nullptr, nullptr, 0, st)));
      QBG_TRY(run_x<T>(p, false, ns, st));
    }
    QBG_TRY((run_z_fwd<T, 0>(p, c + (size_t)s0 * ldc, ldc, ns, nullptr, 0, 0, nullptr, 0, zero,
                             st)));
  }
  return QBG_OK;
}

template <typename T>
qbg_status density(qbg_plan* p, const double2* c, int ldc, int nst, const double* d_w,
                   double* rho, cudaStream_t st) {
  const int ch = std::max(1, std::min(p->chunk, nst));
  QBG_TRY(ensure_scratch<T>(p, ch));
  if (nst == 0) {
    QBG_CUDA(cudaMemsetAsync(rho, 0, sizeof(double) * p->N, st));
    return QBG_OK;
  }
  // one density slot per state of a chunk (grid-sized), summed at the end
  QBG_TRY(ensure((void**)&p->d_rho_slots, &p->rho_slots_bytes,
                 sizeof(double) * (size_t)p->N * ch));
  size_t xy_smem = 0;
  const bool plane = plane_applies(p, std::is_same<T, float>::value);
  const int G = plane ? 0 : xy_density_group<T>(p, &xy_smem);
  for (int s0 = 0; s0 < nst; s0 += ch) {
    const int ns = std::min(ch, nst - s0);
    QBG_TRY(run_z_bwd<T>(p, c + (size_t)s0 * ldc, ldc, ns, st));
    if (plane) {
      if constexpr (!std::is_same<T, float>::value)
        QBG_TRY(plane_density<T>(p, ns, d_w + s0, s0 > 0 ? 1 : 0, p->d_rho_slots, st));
    } else if (G) {
      if constexpr (!std::is_same<T, float>::value)
        QBG_TRY(run_xy_density<T>(p, ns, d_w + s0, s0 > 0 ? 1 : 0, G, xy_smem, st));
    } else {
      QBG_TRY(run_x<T>(p, true, ns, st));
      QBG_TRY((run_y<T, Y_DENSITY>(p, ns, nullptr, d_w + s0, p->d_rho_slots, s0 > 0 ? 1 : 0,
                                   st)));
    }
  }
  {
    PhaseTimer pt(p, PH_Y_DENSITY, st);
    if ((G || plane) && std::is_same<T, df32>::value)
      k_sum_slots<df32><<<2 * 152 * 4, 256, 0, st>>>((const df32*)p->d_rho_slots, ch, p->N, rho);
    else
      k_sum_slots<double><<<2 * 152 * 4, 256, 0, st>>>(p->d_rho_slots, ch, p->N, rho);
    QBG_LAUNCHED(p);
  }
  return QBG_OK;
}

// Backward transform with caller-provided scratch (Z for chunk*n2*nrods,
// Y for chunk*n2*nband*n0 complex elements of type T); allocates nothing.
// The same launchers (thread counts, shared memory) as backward().
template <typename T>
qbg_status backward_scratch(qbg_plan* p, const double2* c, int ldc, double2* f, int nb,
                            void* Z, void* Y, int chunk, cudaStream_t st) {
  for (int s0 = 0; s0 < nb; s0 += chunk) {
    const int ns = std::min(chunk, nb - s0);
    QBG_TRY(run_z_bwd<T>(p, c + (size_t)s0 * ldc, ldc, ns, st, Z));
    QBG_TRY(run_x<T>(p, true, ns, st, Z, Y));
    QBG_TRY(big_prime(p->len[1])
                ? (run_y_<T, Y_BWD_STORE, true>(p, ns, f + (size_t)s0 * p->N, nullptr, nullptr,
                                                0, st, Y))
                : (run_y_<T, Y_BWD_STORE, false>(p, ns, f + (size_t)s0 * p->N, nullptr, nullptr,
                                                 0, st, Y)));
  }
  return QBG_OK;
}

template qbg_status backward_scratch<double>(qbg_plan*, const double2*, int, double2*, int, void*,
                                             void*, int, cudaStream_t);

template qbg_status local_hpsi<double>(qbg_plan*, const double2*, int, double2*, int, bool,
                                       double2*, int, double2, cudaStream_t);
template qbg_status local_hpsi<float>(qbg_plan*, const double2*, int, double2*, int, bool,
                                      double2*, int, double2, cudaStream_t);
template qbg_status backward<double>(qbg_plan*, const double2*, int, double2*, int, cudaStream_t);
template qbg_status backward<float>(qbg_plan*, const double2*, int, double2*, int, cudaStream_t);
template qbg_status backward<df32>(qbg_plan*, const double2*, int, double2*, int, cudaStream_t);
template qbg_status forward<double>(qbg_plan*, double2*, double2*, int, int, cudaStream_t);
template qbg_status density<double>(qbg_plan*, const double2*, int, int, const double*, double*,
                                    cudaStream_t);
template qbg_status density<float>(qbg_plan*, const double2*, int, int, const double*, double*,
                                   cudaStream_t);
template qbg_status local_hpsi<df32>(qbg_plan*, const double2*, int, double2*, int, bool,
                                     double2*, int, double2, cudaStream_t);
template qbg_status density<df32>(qbg_plan*, const double2*, int, int, const double*, double*,
                                  cudaStream_t);

}  // namespace qbg
