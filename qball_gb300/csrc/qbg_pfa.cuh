// qbg_pfa.cuh -- prime-factor (Good-Thomas) transforms of lines whose length
// splits into two coprime factors, N = N1 * N2, gcd(N1, N2) = 1.
//
// With the input map n = (N2 n1 + N1 n2) mod N and the output map
// k = (K1 k1 + K2 k2) mod N (K1 = 1 mod N1, 0 mod N2; K2 = 0 mod N1,
// 1 mod N2), exp(2 pi i n k / N) = exp(2 pi i n1 k1 / N1) exp(2 pi i n2 k2 / N2),
// so the transform is N2 transforms of length N1 followed by N1 of length N2
// with no twiddle factors between them (Good 1958, Thomas 1963).  Against the
// three-pass mixed-radix Stockham transform this removes every twiddle
// product and one shared-memory round trip: 120 = 8 x 15 takes two passes
// of unrolled register codelets (15 = 3 x 5 is itself prime-factor).
//
// Pass 1 works in place on the input slots (each (line, n2) item owns the
// slots n = N2 n1 + N1 n2); pass 2 reads those slots and writes the result in
// natural order into the second buffer.  Items are numbered line-fastest so
// that consecutive threads touch consecutive lines: with an odd line stride
// every shared-memory access of a warp is free of bank conflicts.
#pragma once
// included at the end of qbg_fft_engine.cuh

namespace qbg {

constexpr int pfa_inv(int a, int m) {  // a^-1 mod m, gcd(a, m) = 1
  int r = 1;
  while ((a * r) % m != 1) ++r;
  return r;
}
constexpr int pfa_gcd(int a, int b) { return b == 0 ? a : pfa_gcd(b, a % b); }

template <int N1, int N2> struct PfaMap {
  static_assert(pfa_gcd(N1, N2) == 1, "prime-factor split needs coprime factors");
  static constexpr int N = N1 * N2;
  static constexpr int K1 = N2 * pfa_inv(N2 % N1, N1);  // 1 mod N1, 0 mod N2
  static constexpr int K2 = N1 * pfa_inv(N1 % N2, N2);  // 0 mod N1, 1 mod N2
};

// pass 1 of one (line, n2) item: length-N1 transform of x[N2 n1 + N1 n2]
template <int N1, int N2, int S, typename C>
__host__ __device__ __forceinline__ void pfa_item1(C* line, int n2) {
  constexpr int N = N1 * N2;
  const int base = N1 * n2;  // < N
  C v[N1];
#pragma unroll
  for (int a = 0; a < N1; ++a) {
    int i = base + N2 * a;
    i = i >= N ? i - N : i;
    v[a] = line[i];
  }
  dft_r<N1, S>(v, (const C*)nullptr, 0, 0, 0);
#pragma unroll
  for (int a = 0; a < N1; ++a) {
    int i = base + N2 * a;
    i = i >= N ? i - N : i;
    line[i] = v[a];
  }
}

// pass 2 of one (line, k1) item: length-N2 transform over n2 of the pass-1
// results, written to natural order k = K1 k1 + K2 k2 (mod N)
template <int N1, int N2, int S, typename C>
__host__ __device__ __forceinline__ void pfa_item2(const C* src, C* dst, int k1) {
  using M = PfaMap<N1, N2>;
  constexpr int N = M::N;
  const int base = N2 * k1;  // < N
  C v[N2];
#pragma unroll
  for (int b = 0; b < N2; ++b) {
    int i = base + N1 * b;
    i = i >= N ? i - N : i;
    v[b] = src[i];
  }
  dft_r<N2, S>(v, (const C*)nullptr, 0, 0, 0);
  const int obase = (M::K1 * k1) % N;
#pragma unroll
  for (int b = 0; b < N2; ++b) {
    int i = obase + (M::K2 * b) % N;
    i = i >= N ? i - N : i;
    dst[i] = v[b];
  }
}

// Transform of nlines lines of length N1*N2 held in A (line stride ls).
// When every pass-2 item has a thread of its own (nlines * N1 <= blockDim.x)
// the result is left in A (each thread holds its item across a barrier) and
// B is not touched; otherwise it is left in B.  Ends with __syncthreads().
template <int N1, int N2, int S, typename T>
__device__ __forceinline__ cplx<T>* pfa_lines(cplx<T>* A, cplx<T>* B, int nlines, int ls) {
  using C = cplx<T>;
  using M = PfaMap<N1, N2>;
  const int items1 = nlines * N2;
  for (int it = threadIdx.x; it < items1; it += blockDim.x) {
    const int n2 = it / nlines;
    const int line = it - n2 * nlines;
    pfa_item1<N1, N2, S>(A + line * ls, n2);
  }
  __syncthreads();
  const int items2 = nlines * N1;
  if (items2 <= (int)blockDim.x) {
    const bool act = (int)threadIdx.x < items2;
    const int k1 = threadIdx.x / nlines;
    C* ln = A + (threadIdx.x - k1 * nlines) * ls;
    C v[N2];
    if (act) {
      const int base = N2 * k1;
#pragma unroll
      for (int b = 0; b < N2; ++b) {
        int i = base + N1 * b;
        i = i >= M::N ? i - M::N : i;
        v[b] = ln[i];
      }
      dft_r<N2, S>(v, (const C*)nullptr, 0, 0, 0);
    }
    __syncthreads();
    if (act) {
      const int obase = (M::K1 * k1) % M::N;
#pragma unroll
      for (int b = 0; b < N2; ++b) {
        int i = obase + (M::K2 * b) % M::N;
        i = i >= M::N ? i - M::N : i;
        ln[i] = v[b];
      }
    }
    __syncthreads();
    return A;
  }
  for (int it = threadIdx.x; it < items2; it += blockDim.x) {
    const int k1 = it / nlines;
    const int line = it - k1 * nlines;
    pfa_item2<N1, N2, S>(A + line * ls, B + line * ls, k1);
  }
  __syncthreads();
  return B;
}

// ---- 120 = 8 x 3 x 5 as three prime-factor passes ------------------------
// Nesting 15 = 3 x 5 inside 120 = 8 x 15 gives the input slot of (n1, a, b),
// n1 < 8, a < 3, b < 5, as (15 n1 + 40 a + 24 b) mod 120 and the output index
// of (k1, ka, kb) as (105 k1 + 40 ka + 96 kb) mod 120 (k = k1 mod 8,
// k = 10 ka + 6 kb mod 15).  The 3-point and 5-point passes run in place on
// the slots (40 and 24 items per line); the 8-point pass (15 items per line)
// is left to the caller, which decides where its outputs go.  Against the
// two-pass split the longest per-item codelet drops from 1500 to 432
// double-float instructions, so more threads share every pass.
__host__ __device__ __forceinline__ int pfa120_slot(int n1, int a, int b) {
  return (15 * n1 + 40 * a + 24 * b) % 120;
}
__host__ __device__ __forceinline__ int pfa120_out(int k1, int ka, int kb) {
  return (105 * k1 + 40 * ka + 96 * kb) % 120;
}
// x mod 120 for 0 <= x < 240
__device__ __forceinline__ int mod120(int x) { return x >= 120 ? x - 120 : x; }
// (q, r) = divmod(it, n) with inv = 1/n in FP32 (it < 2^20, n <= 4096)
__device__ __forceinline__ int divf(int it, float inv) { return (int)(((float)it + 0.5f) * inv); }

// the 3-point and 5-point passes over nl lines (stride ls); ends with a
// barrier.  Slot indices advance by +40 (a) and +24 (b) modulo 120.
template <int S, typename C>
__device__ __forceinline__ void pfa120_ab(C* L, int ls, int nl) {
  const float inl = 1.f / (float)nl;
  for (int it = threadIdx.x; it < nl * 40; it += blockDim.x) {
    const int j = divf(it, inl), line = it - j * nl;  // j = 5 n1 + b
    const int n1 = divf(j, 0.2f), b = j - 5 * n1;
    C* ln = L + line * ls;
    const int i0 = pfa120_slot(n1, 0, b), i1 = mod120(i0 + 40), i2 = mod120(i1 + 40);
    C v[3] = {ln[i0], ln[i1], ln[i2]};
    dft3<S>(v);
    ln[i0] = v[0];
    ln[i1] = v[1];
    ln[i2] = v[2];
  }
  __syncthreads();
  for (int it = threadIdx.x; it < nl * 24; it += blockDim.x) {
    const int j = divf(it, inl), line = it - j * nl;  // j = 3 n1 + ka
    const int n1 = divf(j, 1.f / 3.f), ka = j - 3 * n1;
    C* ln = L + line * ls;
    int idx[5];
    idx[0] = pfa120_slot(n1, ka, 0);
#pragma unroll
    for (int b = 1; b < 5; ++b) idx[b] = mod120(idx[b - 1] + 24);
    C v[5];
#pragma unroll
    for (int b = 0; b < 5; ++b) v[b] = ln[idx[b]];
    dft5<S>(v);
#pragma unroll
    for (int b = 0; b < 5; ++b) ln[idx[b]] = v[b];
  }
  __syncthreads();
}

// the 8-point pass of item (ka, kb) of one line: v[k1] is the output at
// pfa120_out(k1, ka, kb) (outputs advance by +105 modulo 120)
template <int S, typename C>
__device__ __forceinline__ void pfa120_c(const C* ln, int ka, int kb, C* v) {
  int i = pfa120_slot(0, ka, kb);
#pragma unroll
  for (int n1 = 0; n1 < 8; ++n1) {
    v[n1] = ln[i];
    i = mod120(i + 15);
  }
  dft8<S>(v);
}

// whole transform of nl <= blockDim.x / 15 lines in place (the 8-point pass
// holds its item in registers across a barrier); ends with a barrier
template <int S, typename C>
__device__ __forceinline__ void pfa120_lines(C* L, int ls, int nl) {
  pfa120_ab<S>(L, ls, nl);
  const bool act = (int)threadIdx.x < nl * 15;
  const int j = divf(threadIdx.x, 1.f / (float)nl), line = threadIdx.x - j * nl;  // j = 5 ka + kb
  const int ka = divf(j, 0.2f), kb = j - 5 * ka;
  C v[8];
  if (act) pfa120_c<S>(L + line * ls, ka, kb, v);
  __syncthreads();
  if (act) {
    C* ln = L + line * ls;
    int o = pfa120_out(0, ka, kb);
#pragma unroll
    for (int k1 = 0; k1 < 8; ++k1) {
      ln[o] = v[k1];
      o = mod120(o + 105);
    }
  }
  __syncthreads();
}

// ---- 120 points in place and in order ------------------------------------
// The same Ruritanian map n = (15 n1 + 40 a + 24 b) mod 120 (n1 < 8, a < 3,
// b < 5) for input and output (Burrus and Eschenbacher, 1981): n k = 105 n1
// k1 + 40 a ka + 96 b kb (mod 120), so for the direction s the transform is
// a 3-point DFT over a with exp(s 2 pi i / 3), a 5-point DFT over b with
// exp(s 2 pi i 4/5) = exp(-s 2 pi i / 5) and an 8-point DFT over n1 with
// exp(s 2 pi i 7/8) = exp(-s 2 pi i / 8).  Each item of each pass reads
// and writes the same slots: items are independent, the passes commute, and
// nothing is held in registers across a barrier.
__host__ __device__ __forceinline__ int pl_m120(int x) { return x >= 120 ? x - 120 : x; }

// slots of item j of in-place pass P (0: 3-point over a, 1: 5-point over b, 2:
// 8-point over n1): i[0] first, consecutive slots STEP apart mod 120
template <int P> struct PlPass;
template <> struct PlPass<0> {  // j = 5 n1 + b < 40
  static constexpr int R = 3, NI = 40, STEP = 40;
  __device__ __forceinline__ static int base(int j) {
    const int n1 = j / 5, b = j - 5 * n1;
    return pl_m120(15 * n1 + 24 * b);
  }
};
template <> struct PlPass<1> {  // j = 3 n1 + a < 24
  static constexpr int R = 5, NI = 24, STEP = 24;
  __device__ __forceinline__ static int base(int j) {
    const int n1 = j / 3, a = j - 3 * n1;
    return pl_m120(15 * n1 + 40 * a);
  }
};
template <> struct PlPass<2> {  // j = 5 a + b < 15
  static constexpr int R = 8, NI = 15, STEP = 15;
  __device__ __forceinline__ static int base(int j) {
    const int a = j / 5, b = j - 5 * a;
    return pl_m120(40 * a + 24 * b);
  }
};

template <int P> __device__ __forceinline__ void pl_slots(int j, int* i) {
  i[0] = PlPass<P>::base(j);
#pragma unroll
  for (int k = 1; k < PlPass<P>::R; ++k) i[k] = pl_m120(i[k - 1] + PlPass<P>::STEP);
}

// the pass' codelet for direction S (+1 backward, -1 forward)
template <int P, int S, typename C> __device__ __forceinline__ void pl_dft(C* v) {
  if constexpr (P == 0) dft3<S>(v);
  else if constexpr (P == 1) dft5<-S>(v);
  else dft8<-S>(v);
}

// one item of pass P on the line at ln (element stride ST)
template <int P, int S, int ST, typename C>
__device__ __forceinline__ void pl_item(C* ln, int j) {
  constexpr int R = PlPass<P>::R;
  int i[R];
  pl_slots<P>(j, i);
  C v[R];
#pragma unroll
  for (int k = 0; k < R; ++k) v[k] = ln[i[k] * ST];
  pl_dft<P, S>(v);
#pragma unroll
  for (int k = 0; k < R; ++k) ln[i[k] * ST] = v[k];
}

// all three in-place passes (direction S) over nl lines of 120 points, line
// stride ls, lines fastest across threads; ends with a barrier
template <int S, typename C>
__device__ __forceinline__ void pfa120_inplace_lines(C* L, int ls, int nl) {
  const float inl = 1.f / (float)nl;
  for (int it = threadIdx.x; it < nl * PlPass<0>::NI; it += blockDim.x) {
    const int j = divf(it, inl), line = it - j * nl;
    pl_item<0, S, 1>(L + line * ls, j);
  }
  __syncthreads();
  for (int it = threadIdx.x; it < nl * PlPass<1>::NI; it += blockDim.x) {
    const int j = divf(it, inl), line = it - j * nl;
    pl_item<1, S, 1>(L + line * ls, j);
  }
  __syncthreads();
  for (int it = threadIdx.x; it < nl * PlPass<2>::NI; it += blockDim.x) {
    const int j = divf(it, inl), line = it - j * nl;
    pl_item<2, S, 1>(L + line * ls, j);
  }
  __syncthreads();
}

// prime-factor split used for length n (0: none; the Stockham engine runs)
__host__ __device__ inline int pfa_split(int n) {
  switch (n) {
    case 120: return 8;   // 8 x 15
    case 48: return 16;   // 16 x 3
    case 40: return 8;    // 8 x 5
    case 72: return 8;    // 8 x 9
    case 80: return 16;   // 16 x 5
    case 144: return 16;  // 16 x 9
    default: return 0;
  }
}

// Dispatch on the supported lengths; returns nullptr when n has no split.
template <int S, typename T>
__device__ cplx<T>* pfa_dispatch(cplx<T>* A, cplx<T>* B, int nlines, int ls, int n) {
  switch (n) {
    case 120: return pfa_lines<8, 15, S, T>(A, B, nlines, ls);
    case 48: return pfa_lines<16, 3, S, T>(A, B, nlines, ls);
    case 40: return pfa_lines<8, 5, S, T>(A, B, nlines, ls);
    case 72: return pfa_lines<8, 9, S, T>(A, B, nlines, ls);
    case 80: return pfa_lines<16, 5, S, T>(A, B, nlines, ls);
    case 144: return pfa_lines<16, 9, S, T>(A, B, nlines, ls);
    default: return nullptr;
  }
}

}  // namespace qbg
