// qbg_lanefft.cuh -- register-resident 1-D FFTs with warp-shuffle butterflies.
//
// A line of length n = A*B is held by a group of B consecutive lanes of a
// warp (B = 8 or 16), A complex values per lane.  Two layouts:
//   L1: lane b, register a  <->  index j = b + B*a
//   L2: lane b, register a  <->  index k = a + A*rev(b)   (rev: bit reversal
//                                                         of b over log2 B bits)
// regs_then_lanes maps L1 -> L2: an A-point DFT in registers, the twiddle
// w_n^{b k_a}, then a B-point decimation-in-frequency network across the
// lanes (one shuffle per value and stage; the outputs land bit-reversed).
// lanes_then_regs maps L2 -> L1: a decimation-in-time network across the
// lanes (bit-reversed in, natural out), the twiddle w_n^{j_a k_b}, then the
// A-point DFT in registers.  A backward transform, a pointwise product and a
// forward transform therefore chain with no data exchange between them.
// Derivation (Cooley-Tukey four-step): with j = b + B a and k = k_a + A k_b,
// w_n^{jk} = w_A^{a k_a} w_n^{b k_a} w_B^{b k_b}; the mirror split
// j = j_a + A j_b, k = k_b + B k_a gives the second map.
#pragma once
#include "qbg_fft_engine.cuh"

namespace qbg {

template <int B> __device__ __forceinline__ int lane_rev(int b) {
  if (B == 8) return ((b & 1) << 2) | (b & 2) | ((b >> 2) & 1);
  // B == 16
  return ((b & 1) << 3) | ((b & 2) << 1) | ((b >> 1) & 2) | ((b >> 3) & 1);
}

template <typename C> __device__ __forceinline__ C shfl_xor_c(C v, int m);
template <> __device__ __forceinline__ double2 shfl_xor_c(double2 v, int m) {
  return make_double2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}
template <> __device__ __forceinline__ float2 shfl_xor_c(float2 v, int m) {
  return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}
template <> __device__ __forceinline__ df32c shfl_xor_c(df32c v, int m) {
  df32c r;
  r.x.hi = __shfl_xor_sync(0xffffffffu, v.x.hi, m);
  r.x.lo = __shfl_xor_sync(0xffffffffu, v.x.lo, m);
  r.y.hi = __shfl_xor_sync(0xffffffffu, v.y.hi, m);
  r.y.lo = __shfl_xor_sync(0xffffffffu, v.y.lo, m);
  return r;
}

// A-point DFT in registers for the supported A
template <int A, int S, typename C> __device__ __forceinline__ void dft_regs(C* v) {
  if constexpr (A == 2) dft2<S>(v);
  else if constexpr (A == 3) dft3<S>(v);
  else if constexpr (A == 4) dft4<S>(v);
  else if constexpr (A == 5) dft5<S>(v);
  else if constexpr (A == 6) dft6<S>(v);
  else if constexpr (A == 8) dft8<S>(v);
  else if constexpr (A == 9) dft9<S>(v);
  else if constexpr (A == 10) dft10<S>(v);
  else if constexpr (A == 12) dft12<S>(v);
  else if constexpr (A == 15) dft15<S>(v);
  else if constexpr (A == 16) dft16<S>(v);
}

// twiddle table access: W[m] = exp(-2 pi i m / n) in shared memory; S > 0
// uses the conjugate
template <int S, typename C> __device__ __forceinline__ C twmul(C v, const C* W, int m) {
  const C w = W[m];
  return S > 0 ? cmulc(v, w) : cmul(v, w);
}

// L1 -> L2.  b: lane index within the group.  Wn: n-entry table
// exp(-2 pi i m / n) (w_B^m is Wn[m * n / B]).
template <int S, int A, int B, typename C>
__device__ __forceinline__ void regs_then_lanes(C* v, int b, const C* Wn) {
  constexpr int n = A * B;
  dft_regs<A, S>(v);
  if (b) {
#pragma unroll
    for (int a = 1; a < A; ++a) v[a] = twmul<S>(v[a], Wn, (b * a) % n);
  }
  // decimation in frequency across the lanes
#pragma unroll
  for (int h = B / 2; h >= 1; h >>= 1) {
    const bool upper = (b & h) != 0;
    const C w = Wn[(b & (h - 1)) * (B / (2 * h)) * (n / B)];
#pragma unroll
    for (int a = 0; a < A; ++a) {
      const C p = shfl_xor_c(v[a], h);
      if (!upper) {
        v[a] = cadd(v[a], p);
      } else {
        const C d = csub(p, v[a]);
        v[a] = S > 0 ? cmulc(d, w) : cmul(d, w);
      }
    }
  }
}

// L2 -> L1
template <int S, int A, int B, typename C>
__device__ __forceinline__ void lanes_then_regs(C* v, int b, const C* Wn) {
  constexpr int n = A * B;
  // decimation in time across the lanes: bit-reversed in, natural out
#pragma unroll
  for (int h = 1; h <= B / 2; h <<= 1) {
    const bool upper = (b & h) != 0;
    const C w = Wn[(b & (h - 1)) * (B / (2 * h)) * (n / B)];
#pragma unroll
    for (int a = 0; a < A; ++a) {
      const C t = upper ? (S > 0 ? cmulc(v[a], w) : cmul(v[a], w)) : v[a];
      const C p = shfl_xor_c(t, h);
      v[a] = upper ? csub(p, t) : cadd(t, p);
    }
  }
  if (b) {
#pragma unroll
    for (int a = 1; a < A; ++a) v[a] = twmul<S>(v[a], Wn, (a * b) % n);
  }
  dft_regs<A, S>(v);
}

}  // namespace qbg
