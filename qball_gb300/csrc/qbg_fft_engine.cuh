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

template <typename C> __host__ __device__ __forceinline__ C cmk(decltype(C::x) x, decltype(C::x) y) {
  C c; c.x = x; c.y = y; return c;
}
template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) { return cmk<C>(a.x + b.x, a.y + b.y); }
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) { return cmk<C>(a.x - b.x, a.y - b.y); }
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
  return cmk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename C> __host__ __device__ __forceinline__ C cmulc(C a, C b) {  // a * conj(b)
  return cmk<C>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
// multiply by S*i : S=+1 -> i*(x+iy) = (-y, x); S=-1 -> (y, -x)
template <int S, typename C> __host__ __device__ __forceinline__ C cmul_si(C a) {
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
  float inv_m[kMaxPass];   // 1 / (n / radix)
  float inv_ns[kMaxPass];  // 1 / ns
  int ntw;                 // twiddle table length
  const cplx<T>* tw;    // exp(-2 pi i r k / (ns*radix)), k<ns, r<radix
  const cplx<T>* gtab;  // exp(-2 pi i m / p) for the direct-DFT primes
  const cplx<T>* root;  // exp(-2 pi i m / n), m < n
  int goff7, goff11, goff13;
  int pfa;  // non-zero: n = pfa * (n / pfa) runs as a prime-factor transform
};

constexpr int kGtab = 31;  // 7 + 11 + 13 direct-DFT roots

// floor(a / b) for 0 <= a < 2^20 and 1 <= b <= 2^12 with inv = 1/b rounded
// to FP32: the product's error is far below the gap to the next integer
__device__ __forceinline__ int fdiv(int a, float inv) {
  return (int)(((float)a + 0.5f) * inv);
}

// Copies the length's twiddle tables into shared memory (dst holds
// ntw + kGtab entries) and returns a view that reads them from there.  The
// caller synchronises before the first pass.
template <typename T>
__device__ __forceinline__ FFTLen<T> stage_twiddles(const FFTLen<T>& d, cplx<T>* dst, bool bigp) {
  if (d.pfa) return d;  // prime-factor lengths use no twiddle table
  for (int i = threadIdx.x; i < d.ntw; i += blockDim.x) dst[i] = d.tw[i];
  if (bigp)
    for (int i = threadIdx.x; i < kGtab; i += blockDim.x) dst[d.ntw + i] = d.gtab[i];
  FFTLen<T> v = d;
  v.tw = dst;
  if (bigp) v.gtab = dst + d.ntw;
  return v;
}

// ---------------------------------------------------------------- codelets
template <int S, typename C> __host__ __device__ __forceinline__ void dft2(C* v) {
  C a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

// x/2 (exact): a plain product for float/double, component scaling for
// double-float
template <typename T> __host__ __device__ __forceinline__ T half_of(T x) { return x * T(0.5); }
template <> __host__ __device__ __forceinline__ df32 half_of<df32>(df32 x) {
  return df_scale2(x, 0.5f);
}

template <int S, typename C> __host__ __device__ __forceinline__ void dft3(C* v) {
  using T = decltype(C::x);
  const T h = T(0.86602540378443864676372317075293618);  // sin(2 pi/3)
  C t1 = cadd(v[1], v[2]);
  C t2 = cmk<C>(v[0].x - half_of(t1.x), v[0].y - half_of(t1.y));
  C d = csub(v[1], v[2]);
  C t3 = cmul_si<S>(cmk<C>(h * d.x, h * d.y));
  v[0] = cadd(v[0], t1);
  v[1] = cadd(t2, t3);
  v[2] = csub(t2, t3);
}

template <int S, typename C> __host__ __device__ __forceinline__ void dft4(C* v) {
  C a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
  C c = cadd(v[1], v[3]), d = cmul_si<S>(csub(v[1], v[3]));
  v[0] = cadd(a, c);
  v[2] = csub(a, c);
  v[1] = cadd(b, d);
  v[3] = csub(b, d);
}

template <int S, typename C> __host__ __device__ __forceinline__ void dft5(C* v) {
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

template <int S, typename C> __host__ __device__ __forceinline__ void dft8(C* v) {
  using T = decltype(C::x);
  const T r2 = T(0.70710678118654752440084436210484904);
  C e[4] = {v[0], v[2], v[4], v[6]};
  C o[4] = {v[1], v[3], v[5], v[7]};
  dft4<S>(e);
  dft4<S>(o);
  // o1 *= (1+Si)/sqrt2, o2 *= S i, o3 *= (-1+Si)/sqrt2 (S = +-1 folded into
  // the sums, no multiplication by S)
  C x = o[1];
  if (S > 0)
    o[1] = cmk<C>(r2 * (x.x - x.y), r2 * (x.y + x.x));
  else
    o[1] = cmk<C>(r2 * (x.x + x.y), r2 * (x.y - x.x));
  o[2] = cmul_si<S>(o[2]);
  x = o[3];
  if (S > 0)
    o[3] = cmk<C>(-(r2 * (x.x + x.y)), r2 * (x.x - x.y));
  else
    o[3] = cmk<C>(r2 * (x.y - x.x), -(r2 * (x.x + x.y)));
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = cadd(e[k], o[k]);
    v[k + 4] = csub(e[k], o[k]);
  }
}

// direct DFT for a small prime p with table g[m] = exp(-2 pi i m/p)
template <int P, int S, typename C>
__host__ __device__ __forceinline__ void dftp(C* v, const C* g) {
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

// multiply by the constant exp(S*2*pi*i*e/n) given as (c, s) = (cos, sin)
template <int S, typename C>
__host__ __device__ __forceinline__ C cmul_root(C a, double c, double sn) {
  using T = decltype(C::x);
  const T cr = T(c), ci = T(S * sn);
  return cmk<C>(a.x * cr - a.y * ci, a.x * ci + a.y * cr);
}

// 16 = 4 x 4: X[c+4d] = sum_b W4^{bd} W16^{bc} sum_a x[4a+b] W4^{ac}
template <int S, typename C> __host__ __device__ __forceinline__ void dft16(C* v) {
  const double c1 = 0.92387953251128675612818318939678829, s1 = 0.38268343236508977172845998403039887;
  const double r2 = 0.70710678118654752440084436210484904;
  C y[4][4];
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    C t[4] = {v[b], v[4 + b], v[8 + b], v[12 + b]};
    dft4<S>(t);
#pragma unroll
    for (int c = 0; c < 4; ++c) y[b][c] = t[c];
  }
  // twiddles W16^{bc}
  y[1][1] = cmul_root<S>(y[1][1], c1, s1);
  y[1][2] = cmul_root<S>(y[1][2], r2, r2);
  y[1][3] = cmul_root<S>(y[1][3], s1, c1);
  y[2][1] = cmul_root<S>(y[2][1], r2, r2);
  y[2][2] = cmul_si<S>(y[2][2]);
  y[2][3] = cmul_root<S>(y[2][3], -r2, r2);
  y[3][1] = cmul_root<S>(y[3][1], s1, c1);
  y[3][2] = cmul_root<S>(y[3][2], -r2, r2);
  y[3][3] = cmul_root<S>(y[3][3], -c1, -s1);
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    C t[4] = {y[0][c], y[1][c], y[2][c], y[3][c]};
    dft4<S>(t);
#pragma unroll
    for (int d = 0; d < 4; ++d) v[c + 4 * d] = t[d];
  }
}

// 9 = 3 x 3 with twiddles W9^{bc}
template <int S, typename C> __host__ __device__ __forceinline__ void dft9(C* v) {
  const double c1 = 0.76604444311897803520239265055541667, s1 = 0.64278760968653932632264340990726344;  // 2pi/9
  const double c2 = 0.17364817766693034885171662676931480, s2 = 0.98480775301220805936674302458952301;  // 4pi/9
  const double c4 = -0.93969262078590838405410927732473147, s4 = 0.34202014332566873304409961468225958; // 8pi/9
  C y[3][3];
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    C t[3] = {v[b], v[3 + b], v[6 + b]};
    dft3<S>(t);
#pragma unroll
    for (int c = 0; c < 3; ++c) y[b][c] = t[c];
  }
  y[1][1] = cmul_root<S>(y[1][1], c1, s1);
  y[1][2] = cmul_root<S>(y[1][2], c2, s2);
  y[2][1] = cmul_root<S>(y[2][1], c2, s2);
  y[2][2] = cmul_root<S>(y[2][2], c4, s4);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    C t[3] = {y[0][c], y[1][c], y[2][c]};
    dft3<S>(t);
#pragma unroll
    for (int d = 0; d < 3; ++d) v[c + 3 * d] = t[d];
  }
}

// Good-Thomas prime-factor DFT of N = N1*N2 (coprime): input n = (N2 n1 + N1 n2)
// mod N, output k with k = k1 (mod N1), k = k2 (mod N2) -- a 2-D DFT without
// twiddles.  K1, K2 are the CRT coefficients (k = K1 k1 + K2 k2 mod N).
template <int S, int N1, int N2, int K1, int K2, typename C, typename F1, typename F2>
__host__ __device__ __forceinline__ void dft_pfa(C* v, F1 f1, F2 f2) {
  constexpr int N = N1 * N2;
  C y[N1][N2];
#pragma unroll
  for (int n1 = 0; n1 < N1; ++n1) {
    C t[N2];
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) t[n2] = v[(N2 * n1 + N1 * n2) % N];
    f2(t);
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) y[n1][k2] = t[k2];
  }
#pragma unroll
  for (int k2 = 0; k2 < N2; ++k2) {
    C t[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) t[n1] = y[n1][k2];
    f1(t);
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) v[(K1 * k1 + K2 * k2) % N] = t[k1];
  }
}

template <int S, typename C> __host__ __device__ __forceinline__ void dft15(C* v) {
  dft_pfa<S, 3, 5, 10, 6>(v, [](C* t) { dft3<S>(t); }, [](C* t) { dft5<S>(t); });
}
template <int S, typename C> __host__ __device__ __forceinline__ void dft10(C* v) {
  dft_pfa<S, 2, 5, 5, 6>(v, [](C* t) { dft2<S>(t); }, [](C* t) { dft5<S>(t); });
}
template <int S, typename C> __host__ __device__ __forceinline__ void dft6(C* v) {
  dft_pfa<S, 2, 3, 3, 4>(v, [](C* t) { dft2<S>(t); }, [](C* t) { dft3<S>(t); });
}
template <int S, typename C> __host__ __device__ __forceinline__ void dft12(C* v) {
  dft_pfa<S, 4, 3, 9, 4>(v, [](C* t) { dft4<S>(t); }, [](C* t) { dft3<S>(t); });
}

template <int R, int S, typename C>
__host__ __device__ __forceinline__ void dft_r(C* v, const C* gtab, int g7, int g11, int g13) {
  if constexpr (R == 2) dft2<S>(v);
  else if constexpr (R == 3) dft3<S>(v);
  else if constexpr (R == 4) dft4<S>(v);
  else if constexpr (R == 5) dft5<S>(v);
  else if constexpr (R == 8) dft8<S>(v);
  else if constexpr (R == 16) dft16<S>(v);
  else if constexpr (R == 9) dft9<S>(v);
  else if constexpr (R == 6) dft6<S>(v);
  else if constexpr (R == 10) dft10<S>(v);
  else if constexpr (R == 12) dft12<S>(v);
  else if constexpr (R == 15) dft15<S>(v);
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
  const float inv_m = d.inv_m[p], inv_ns = d.inv_ns[p];
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    const int line = fdiv(it, inv_m);
    const int j = it - line * m;
    const C* s = src + line * ls;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = s[j + r * m];
    const int k = j - fdiv(j, inv_ns) * Ns;
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
template <int S, typename T> __device__ cplx<T>* pfa_dispatch(cplx<T>*, cplx<T>*, int, int, int);

template <int S, typename T, bool BIGP>
__device__ cplx<T>* fft_lines(cplx<T>* A, cplx<T>* B, int nlines, int ls,
                              const FFTLen<T>& d) {
  if constexpr (!BIGP) {
    if (d.pfa) return pfa_dispatch<S, T>(A, B, nlines, ls, d.n);
  }
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

#include "qbg_pfa.cuh"
