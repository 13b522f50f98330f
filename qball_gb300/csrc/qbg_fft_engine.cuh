// qbg_fft_engine.cuh -- batched 1-D complex FFT passes in shared memory.
//
// A CTA holds `nlines` lines of length n (line stride `ls` >= n, padding
// breaks shared-memory bank conflicts) and runs a Stockham auto-sort
// transform over all of them, every thread taking butterflies from every
// line.  Radix-2/3/4/5/8 butterflies are hand-written; 7, 11 and 13 use a
// direct DFT with a small table.  Twiddles come from per-length tables built
// on the host in extended precision (qbg_plan.cu), stored for the
// exp(-i...) sign and conjugated for the backward direction.
//
// Direction convention (same as the reference's cfftm idir):
//   DIR = +1 : backward, y_k = sum_j x_j exp(+2 pi i jk/n)
//   DIR = -1 : forward,  y_k = sum_j x_j exp(-2 pi i jk/n)
#pragma once
#include <cuda_runtime.h>

#include "qbg_df32.cuh"

namespace qbg {

template <typename T> struct cplx_of;
template <> struct cplx_of<double> { using type = double2; };
template <> struct cplx_of<float> { using type = float2; };
template <> struct cplx_of<df32> { using type = df32c; };
template <typename T> using cplx = typename cplx_of<T>::type;

template <typename C> __device__ __forceinline__ C cmk(decltype(C::x) x, decltype(C::x) y) {
  C c; c.x = x; c.y = y; return c;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return cmk<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return cmk<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  return cmk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename C> __device__ __forceinline__ C cmulc(C a, C b) {  // a * conj(b)
  return cmk<C>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
// multiply by S*i : S=+1 -> i*(x+iy) = (-y, x); S=-1 -> (y, -x)
template <int S, typename C> __device__ __forceinline__ C cmul_si(C a) {
  return S > 0 ? cmk<C>(-a.y, a.x) : cmk<C>(a.y, -a.x);
}

constexpr int kMaxPass = 8;

// Device view of one transform length.
template <typename T> struct FFTLen {
  int n;
  int npass;
  int radix[kMaxPass];
  int ns[kMaxPass];     // product of the radices of the passes before
  int twoff[kMaxPass];  // offset of the pass' twiddles in tw
  const cplx<T>* tw;    // exp(-2 pi i r k / (ns*radix)), k<ns, r<radix
  const cplx<T>* gtab;  // exp(-2 pi i m / p) for the direct-DFT primes
  int goff7, goff11, goff13;
};

// ---------------------------------------------------------------- codelets
template <int S, typename C> __device__ __forceinline__ void dft2(C* v) {
  C a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <int S, typename C> __device__ __forceinline__ void dft3(C* v) {
  using T = decltype(C::x);
  const T h = T(0.86602540378443864676372317075293618);  // sin(2 pi/3)
  C t1 = cadd(v[1], v[2]);
  C t2 = cmk<C>(v[0].x - T(0.5) * t1.x, v[0].y - T(0.5) * t1.y);
  C d = csub(v[1], v[2]);
  C t3 = cmul_si<S>(cmk<C>(h * d.x, h * d.y));
  v[0] = cadd(v[0], t1);
  v[1] = cadd(t2, t3);
  v[2] = csub(t2, t3);
}

template <int S, typename C> __device__ __forceinline__ void dft4(C* v) {
  C a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
  C c = cadd(v[1], v[3]), d = cmul_si<S>(csub(v[1], v[3]));
  v[0] = cadd(a, c);
  v[2] = csub(a, c);
  v[1] = cadd(b, d);
  v[3] = csub(b, d);
}

template <int S, typename C> __device__ __forceinline__ void dft5(C* v) {
  using T = decltype(C::x);
  const T c1 = T(0.30901699437494742410229341718281906);   // cos(2 pi/5)
  const T c2 = T(-0.80901699437494742410229341718281906);  // cos(4 pi/5)
  const T s1 = T(0.95105651629515357211643933337938214);   // sin(2 pi/5)
  const T s2 = T(0.58778525229247312916870595463907277);   // sin(4 pi/5)
  C a1 = cadd(v[1], v[4]), a2 = cadd(v[2], v[3]);
  C b1 = csub(v[1], v[4]), b2 = csub(v[2], v[3]);
  C y0 = cadd(v[0], cadd(a1, a2));
  C t1 = cmk<C>(v[0].x + c1 * a1.x + c2 * a2.x, v[0].y + c1 * a1.y + c2 * a2.y);
  C t2 = cmk<C>(v[0].x + c2 * a1.x + c1 * a2.x, v[0].y + c2 * a1.y + c1 * a2.y);
  C u1 = cmul_si<S>(cmk<C>(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y));
  C u2 = cmul_si<S>(cmk<C>(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y));
  v[0] = y0;
  v[1] = cadd(t1, u1);
  v[4] = csub(t1, u1);
  v[2] = cadd(t2, u2);
  v[3] = csub(t2, u2);
}

template <int S, typename C> __device__ __forceinline__ void dft8(C* v) {
  using T = decltype(C::x);
  const T r2 = T(0.70710678118654752440084436210484904);
  C e[4] = {v[0], v[2], v[4], v[6]};
  C o[4] = {v[1], v[3], v[5], v[7]};
  dft4<S>(e);
  dft4<S>(o);
  // o1 *= (1+Si)/sqrt2, o2 *= S i, o3 *= (-1+Si)/sqrt2
  C x = o[1];
  o[1] = cmk<C>(r2 * (x.x - T(S) * x.y), r2 * (x.y + T(S) * x.x));
  o[2] = cmul_si<S>(o[2]);
  x = o[3];
  o[3] = cmk<C>(r2 * (-x.x - T(S) * x.y), r2 * (-x.y + T(S) * x.x));
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = cadd(e[k], o[k]);
    v[k + 4] = csub(e[k], o[k]);
  }
}

// direct DFT for a small prime p with table g[m] = exp(-2 pi i m/p)
template <int P, int S, typename C>
__device__ __forceinline__ void dftp(C* v, const C* g) {
  C y[P];
#pragma unroll
  for (int k = 0; k < P; ++k) {
    C acc = v[0];
#pragma unroll
    for (int j = 1; j < P; ++j) {
      C w = g[(j * k) % P];
      if (S > 0) w.y = -w.y;
      acc = cadd(acc, cmul(v[j], w));
    }
    y[k] = acc;
  }
#pragma unroll
  for (int k = 0; k < P; ++k) v[k] = y[k];
}

template <int R, int S, typename C>
__device__ __forceinline__ void dft_r(C* v, const C* gtab, int g7, int g11, int g13) {
  if constexpr (R == 2) dft2<S>(v);
  else if constexpr (R == 3) dft3<S>(v);
  else if constexpr (R == 4) dft4<S>(v);
  else if constexpr (R == 5) dft5<S>(v);
  else if constexpr (R == 8) dft8<S>(v);
  else if constexpr (R == 7) dftp<7, S>(v, gtab + g7);
  else if constexpr (R == 11) dftp<11, S>(v, gtab + g11);
  else if constexpr (R == 13) dftp<13, S>(v, gtab + g13);
}

// One Stockham pass of radix R over nlines lines: src -> dst.
template <int R, int S, typename T>
__device__ __forceinline__ void fft_pass(const cplx<T>* __restrict__ src,
                                         cplx<T>* __restrict__ dst, int nlines,
                                         int ls, const FFTLen<T>& d, int p) {
  using C = cplx<T>;
  const int n = d.n;
  const int m = n / R;
  const int Ns = d.ns[p];
  const C* tw = d.tw + d.twoff[p];
  const int items = nlines * m;
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    const int line = it / m;
    const int j = it - line * m;
    const C* s = src + line * ls;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = s[j + r * m];
    const int k = j % Ns;
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        C w = tw[k * R + r];
        v[r] = S > 0 ? cmulc(v[r], w) : cmul(v[r], w);
      }
    }
    dft_r<R, S>(v, d.gtab, d.goff7, d.goff11, d.goff13);
    C* o = dst + line * ls + (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) o[r * Ns] = v[r];
  }
}

// Full transform of nlines lines held in A (B is scratch of the same size).
// Returns the buffer that holds the result.  Ends with __syncthreads().
// BIGP selects the build that also carries the 7/11/13 direct DFTs (their
// unrolled bodies raise the register count of every kernel that holds them).
template <int S, typename T, bool BIGP>
__device__ cplx<T>* fft_lines(cplx<T>* A, cplx<T>* B, int nlines, int ls,
                              const FFTLen<T>& d) {
  for (int p = 0; p < d.npass; ++p) {
    switch (d.radix[p]) {
      case 2: fft_pass<2, S, T>(A, B, nlines, ls, d, p); break;
      case 3: fft_pass<3, S, T>(A, B, nlines, ls, d, p); break;
      case 4: fft_pass<4, S, T>(A, B, nlines, ls, d, p); break;
      case 5: fft_pass<5, S, T>(A, B, nlines, ls, d, p); break;
      case 8: fft_pass<8, S, T>(A, B, nlines, ls, d, p); break;
      case 7: if constexpr (BIGP) fft_pass<7, S, T>(A, B, nlines, ls, d, p); break;
      case 11: if constexpr (BIGP) fft_pass<11, S, T>(A, B, nlines, ls, d, p); break;
      case 13: if constexpr (BIGP) fft_pass<13, S, T>(A, B, nlines, ls, d, p); break;
      default: break;
    }
    __syncthreads();
    cplx<T>* t = A;
    A = B;
    B = t;
  }
  return A;
}

}  // namespace qbg
