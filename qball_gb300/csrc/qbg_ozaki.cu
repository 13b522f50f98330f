// qbg_ozaki.cu -- FP64-accurate projector GEMMs on the tensor cores
// (Ozaki scheme) for the plain FP64 form.
//
// The two complex GEMMs of NonLocalPotential::energy (NonLocalPotential.cc:
// 2059-2170, ZGEMM at :2064 and :2165) run as the same real K-major GEMMs as
// the mixed forms (qbg_tc.cu): D[M x N] = A[M x K] B[N x K]^T with the
// interleaved (re, im) operands.  GB300 runs FP64 at ~1 TFLOP/s and FP16
// tensor MMAs at ~1900 TFLOP/s, so the FP64 products are emulated with the
// error-free splitting of Ozaki, Ogita, Oishi and Rump (2012), in the form
// that tensor cores with FP32 accumulation allow (Mukunoki, Ozaki, Ogita and
// Imamura, "DGEMM using Tensor Cores, and Its Accurate and Reproducible
// Versions", ISC 2020):
//
//  * every row of A and of B is scaled by a power of two 2^e (row maximum
//    below 2^e) and written as a fixed-point number with S balanced 7-bit
//    digits: x = sum_{i=1..S} m_i 2^(-7 i), |m_1| <= 128, |m_i| <= 64 (i > 1),
//    rounded at 2^(-7 S - 1) of the row scale (S = 7: 49 bits, S = 6: 42);
//    each digit plane ("slice") is an FP16 matrix of small integers, exact;
//  * a product of two slices sums integers below 2^14 per term, so the
//    FP32 tensor-memory accumulator is exact as long as the sum stays below
//    2^24: every diagonal d = i + j (all slice pairs with the same scale
//    2^(-7 d)) is accumulated over a window of K elements small enough for
//    that bound (512, 448 for d = 8), then read back and folded into a
//    compensated FP32 pair (hi, lo) per output element held in registers;
//  * pairs with i + j > S + 1 are dropped (below the rounding of the
//    digits), so S = 7 runs 28 slice products and S = 6 runs 21.
// The diagonals are processed in groups of at most three, each group one
// sweep over K with only the slices it needs staged in shared memory:
// {2,3,4} (slices 1-3), {5,6,7} (slices 1-6) and {8} (slices 1-7).  The
// three live accumulators take 3 x 128 tensor-memory columns; the fourth
// block of 128 is a spare that rotates, so the MMA warp starts the next
// window while the epilogue reads the last one.
//
// Digits are extracted from the FP64 bit patterns with integer instructions
// (no FP64 arithmetic); the final scaling 2^(eA + eB) is one FP64 multiply.
#include <algorithm>
#include <cstdint>
#include <cuda_fp16.h>
#include <vector>

#include "qbg_internal.h"
#include "qbg_tcgen05.cuh"

namespace qbg {
namespace {

#define QBG_TRY_OZ(x)             \
  do {                            \
    qbg_status s_ = (x);          \
    if (s_ != QBG_OK) return s_;  \
  } while (0)

constexpr int OZ_M = 128;                          // rows per tile (A)
constexpr int OZ_N = 128;                          // rows per tile (B) = MMA N
constexpr int OZ_SMAX = 7;                         // most slices per operand
constexpr int OZ_BLK = 4096;                       // one 128 x 16 FP16 block, bytes
constexpr int OZ_SLOT = 2 * OZ_SMAX * OZ_BLK;      // A slices then B slices: 56 KB
constexpr int OZ_STAGES = 4;
constexpr int OZ_NBUF = 3;                         // accumulators of 128 columns
constexpr int OZ_THREADS = 576;                    // producer, MMA issuer, 16 epilogue warps
constexpr int OZ_EPI = 512;
constexpr int OZ_ECOLS = 32;
constexpr int OZ_SMEM = OZ_STAGES * OZ_SLOT + 1024 + 256;

// One sweep over K: the slice pairs of up to three diagonals, as
// compile-time tables (the MMA loop is unrolled over them).
// Exactness: with |m_1| <= 128 and |m_i| <= 64 the terms of diagonal d are
// bounded per K element by 16384 (d = 2, 3), 20480, 24576, 28672, 32768
// (d = 4..7) and 36864 (d = 8); 512 (448 for d = 8) K elements keep every
// partial sum of the FP32 accumulator below 2^24, hence exact.
template <int G> struct OzG;
// ks: 16-K steps per pipeline stage (the stage holds ks x nsl blocks of A
// and of B; group 0's six MMAs per step are too little work to cover the copy
// latency with one step per stage)
template <> struct OzG<0> {  // diagonals 2, 3, 4: slices 1-3
  static constexpr int nsl = 3, np = 6, nd = 3, win = 32, ks = 2;
  __host__ __device__ static constexpr int diag(int k) { return 2 + k; }
  __host__ __device__ static constexpr int ia(int q) { return q == 0 ? 0 : q == 1 ? 0 : q == 2 ? 1 : q == 3 ? 0 : q == 4 ? 1 : 2; }
  __host__ __device__ static constexpr int acc(int q) { return q == 0 ? 0 : q < 3 ? 1 : 2; }
  __host__ __device__ static constexpr int first(int k) { return k == 0 ? 0 : k == 1 ? 1 : 3; }
};
template <> struct OzG<1> {  // diagonals 5, 6, 7: slices 1-6
  static constexpr int nsl = 6, np = 15, nd = 3, win = 32, ks = 1;
  __host__ __device__ static constexpr int diag(int k) { return 5 + k; }
  __host__ __device__ static constexpr int acc(int q) { return q < 4 ? 0 : q < 9 ? 1 : 2; }
  __host__ __device__ static constexpr int first(int k) { return k == 0 ? 0 : k == 1 ? 4 : 9; }
  __host__ __device__ static constexpr int ia(int q) { return q - first(acc(q)); }
};
template <> struct OzG<2> {  // diagonal 8: slices 1-7
  static constexpr int nsl = 7, np = 7, nd = 1, win = 28, ks = 1;
  __host__ __device__ static constexpr int diag(int) { return 8; }
  __host__ __device__ static constexpr int acc(int) { return 0; }
  __host__ __device__ static constexpr int first(int) { return 0; }
  __host__ __device__ static constexpr int ia(int q) { return q; }
};
// B slice of pair q: the two 0-based slice indices sum to diag - 2
template <class g> __host__ __device__ constexpr int oz_jb(int q) {
  return g::diag(g::acc(q)) - 2 - g::ia(q);
}


// element offset (in halves) of (slice, row, k) in a slice array of nRT row
// tiles and nK16 K steps; one 128 x 16 block is one contiguous image of the
// canonical no-swizzle K-major shared-memory layout (8-row x 16-byte core
// matrices, K-adjacent core matrices 128 B apart, row groups 256 B apart)
__host__ __device__ __forceinline__ size_t oz_index(int sl, int r, int k, int nRT, int nK16) {
  const size_t blk = ((size_t)sl * nRT + (r >> 7)) * nK16 + (k >> 4);
  const int rr = r & 127, kk = k & 15;
  return blk * (OZ_BLK / 2) + (((rr >> 3) * 256 + (kk >> 3) * 128 + (rr & 7) * 16) >> 1) + (kk & 7);
}

// ------------------------------------------------------------ digits
// Row scale exponent from the bit pattern of the row's largest |value|:
// max < 2^e (0 for an all-zero row).
__device__ __forceinline__ int oz_exp(unsigned long long maxbits) {
  const int E = (int)((maxbits >> 52) & 0x7FF);
  return maxbits == 0 ? 0 : (E == 0 ? -1021 : E - 1022);
}

// The nsl balanced 7-bit digits of a * 2^-e (|a| < 2^e): X = round(a
// 2^(7 nsl - e)) from the bit pattern, then least significant digits
// first; m[0] gets the top digit (|m[0]| <= 128).
__device__ __forceinline__ void oz_digits(double a, int e, int nsl, int* m) {
  const long long bits = __double_as_longlong(a);
  const int E = (int)((bits >> 52) & 0x7FF);
  long long M = bits & 0xFFFFFFFFFFFFFll;
  int ex = E;
  if (E == 0) ex = 1; else M |= 0x10000000000000ll;
  // |a| = M 2^(ex - 1075); X = M 2^(ex - 1075 + 7 nsl - e)
  const int sh = ex - 1075 + 7 * nsl - e;
  long long X;
  if (M == 0 || sh < -62) X = 0;
  else if (sh >= 0) X = M << (sh > 10 ? 10 : sh);  // |a| < 2^e keeps sh <= -4
  else X = (M + (1ll << (-sh - 1))) >> (-sh);
  if (bits < 0) X = -X;
#pragma unroll
  for (int i = OZ_SMAX - 1; i >= 1; --i) {
    if (i < nsl) {
      const int d = (int)((X + 64) & 127) - 64;
      m[i] = d;
      X = (X - d) >> 7;
    } else {
      m[i] = 0;
    }
  }
  m[0] = (int)X;
}

// maxima of |re|, |im| of the rows of x[n][0..ncols) as bit patterns
// (integer atomicMax; non-negative doubles order like their bits)
__global__ void k_oz_rowmax(const double2* __restrict__ x, int ld, int ncols,
                            unsigned long long* __restrict__ rmax) {
  __shared__ unsigned long long red[256];
  const int n = blockIdx.y;
  const unsigned long long mask = 0x7FFFFFFFFFFFFFFFull;
  unsigned long long m = 0;
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ncols; g += gridDim.x * blockDim.x) {
    const double2 a = x[(size_t)n * ld + g];
    m = max(m, max((unsigned long long)__double_as_longlong(a.x) & mask,
                   (unsigned long long)__double_as_longlong(a.y) & mask));
  }
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = max(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicMax(rmax + n, red[0]);
}

// per-G maxima over the projectors of the table anl[p][g]
__global__ void k_oz_colmax(const double2* __restrict__ anl, int nproj, int ngw,
                            unsigned long long* __restrict__ gmax) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ngw) return;
  const unsigned long long mask = 0x7FFFFFFFFFFFFFFFull;
  unsigned long long m = 0;
  for (int p = 0; p < nproj; ++p) {
    const double2 a = anl[(size_t)p * ngw + g];
    m = max(m, max((unsigned long long)__double_as_longlong(a.x) & mask,
                   (unsigned long long)__double_as_longlong(a.y) & mask));
  }
  gmax[g] = m;
}

// slices of the interleaved real view of x[n][g] (K = 2 ncols), one row
// exponent per n; 4 complex elements (8 consecutive K, one 16-byte run of a
// block row) per thread
__global__ void k_oz_split_rows(const double2* __restrict__ x, int ld, int ncols,
                                const unsigned long long* __restrict__ rmax, int nsl,
                                __half* __restrict__ Y, int nRT, int nK16,
                                int* __restrict__ eout) {
  const int g0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int n = blockIdx.y;
  const int e = oz_exp(rmax[n]);
  if (g0 == 0) eout[n] = e;
  if (g0 >= ncols) return;
  __align__(16) __half h[OZ_SMAX][8];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int g = g0 + j;
    const double2 a = g < ncols ? x[(size_t)n * ld + g] : make_double2(0.0, 0.0);
    int mr[OZ_SMAX], mi[OZ_SMAX];
    oz_digits(a.x, e, nsl, mr);
    oz_digits(a.y, e, nsl, mi);
#pragma unroll
    for (int s = 0; s < OZ_SMAX; ++s) {
      h[s][2 * j] = __int2half_rn(mr[s]);
      h[s][2 * j + 1] = __int2half_rn(mi[s]);
    }
  }
  for (int s = 0; s < nsl; ++s)
    *reinterpret_cast<uint4*>(Y + oz_index(s, n, 2 * g0, nRT, nK16)) =
        *reinterpret_cast<uint4*>(h[s]);
}

// X1 slices: rows 2p + c, K = 2 ngw, X1[2p][2g] = re, [2p][2g+1] = im,
// [2p+1][2g] = -im, [2p+1][2g+1] = re; one exponent per projector
__global__ void k_oz_split_x1(const double2* __restrict__ anl, int nproj, int ngw,
                              const unsigned long long* __restrict__ pmax, int nsl,
                              __half* __restrict__ X1, int nRT, int nK16,
                              int* __restrict__ eout) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int p = blockIdx.y;
  const int e = oz_exp(pmax[p]);
  if (g == 0) {
    eout[2 * p] = e;
    eout[2 * p + 1] = e;
  }
  if (g >= ngw) return;
  const double2 a = anl[(size_t)p * ngw + g];
  int mr[OZ_SMAX], mi[OZ_SMAX], mn[OZ_SMAX];
  oz_digits(a.x, e, nsl, mr);
  oz_digits(a.y, e, nsl, mi);
  oz_digits(-a.y, e, nsl, mn);
  for (int s = 0; s < nsl; ++s) {
    *reinterpret_cast<__half2*>(X1 + oz_index(s, 2 * p, 2 * g, nRT, nK16)) =
        __halves2half2(__int2half_rn(mr[s]), __int2half_rn(mi[s]));
    *reinterpret_cast<__half2*>(X1 + oz_index(s, 2 * p + 1, 2 * g, nRT, nK16)) =
        __halves2half2(__int2half_rn(mn[s]), __int2half_rn(mr[s]));
  }
}

// X2 = X1^T slices: rows 2g + c, K = 2P, X2[2g][2p] = re, [2g][2p+1] = -im,
// [2g+1][2p] = im, [2g+1][2p+1] = re; one exponent per G
__global__ void k_oz_split_x2(const double2* __restrict__ anl, int nproj, int ngw,
                              const unsigned long long* __restrict__ gmax, int nsl,
                              __half* __restrict__ X2, int nRT, int nK16,
                              int* __restrict__ eout) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int p = blockIdx.y;
  if (g >= ngw) return;
  const int e = oz_exp(gmax[g]);
  if (p == 0) {
    eout[2 * g] = e;
    eout[2 * g + 1] = e;
  }
  const double2 a = anl[(size_t)p * ngw + g];
  int mr[OZ_SMAX], mi[OZ_SMAX], mn[OZ_SMAX];
  oz_digits(a.x, e, nsl, mr);
  oz_digits(a.y, e, nsl, mi);
  oz_digits(-a.y, e, nsl, mn);
  for (int s = 0; s < nsl; ++s) {
    *reinterpret_cast<__half2*>(X2 + oz_index(s, 2 * g, 2 * p, nRT, nK16)) =
        __halves2half2(__int2half_rn(mr[s]), __int2half_rn(mn[s]));
    *reinterpret_cast<__half2*>(X2 + oz_index(s, 2 * g + 1, 2 * p, nRT, nK16)) =
        __halves2half2(__int2half_rn(mi[s]), __int2half_rn(mr[s]));
  }
}

// ------------------------------------------------------------ the GEMM
enum { OZ_OUT_PARTIAL = 0, OZ_OUT_HPSI = 1 };

struct OzArgs {
  const __half* A;   // slices, nsl x nRTa x nK16 blocks
  const __half* B;   // slices, nsl x nRTb x nK16 blocks
  int nRTa, nRTb, nK16;
  int nsl;           // slices per operand (6 or 7)
  int M, N;          // valid rows of A / B
  int k16_per_split; // K steps handled by one CTA (blockIdx.z)
  const int* eA;     // per-row exponents of A (length M)
  const int* eB;     // per-row exponents of B (length N)
  double* out;       // PARTIAL: [split][N][M]; HPSI: complex out, real view
  int ldo;           // HPSI: leading dimension of out in complex elements
  int* status;       // error word (1 = a bounded wait expired)
  int polls;         // poll limit of the pipeline waits (the drains use TC_SPIN)
};

// Shared-memory barriers and the tensor-memory base of one CTA.
struct OzCta {
  unsigned char* smem;
  uint64_t *full, *empty, *accfull, *accempty, *drain;
  volatile int* abort_flag;
  uint32_t tbase;
};

// Producer, one group: one sweep over the CTA's K steps staging the group's
// slices of A and B; q counts stages over all groups.  False on abort.
template <int G>
__device__ __forceinline__ bool oz_produce(const OzArgs& a, const OzCta& c, int mt, int nt,
                                           int ks0, int nks, int& q, int& issued) {
  using g = OzG<G>;
  const size_t sliceA = (size_t)a.nRTa * a.nK16 * (OZ_BLK / 2);
  const size_t sliceB = (size_t)a.nRTb * a.nK16 * (OZ_BLK / 2);
  static_assert(2 * g::ks * g::nsl <= 2 * OZ_SMAX, "stage exceeds its slot");
  static_assert(g::win % g::ks == 0, "windows hold whole stages");
  for (int i = 0; i < nks; i += g::ks, ++q) {
    const int s = q % OZ_STAGES;
    if (q >= OZ_STAGES && !mbar_wait(&c.empty[s], ((q / OZ_STAGES) & 1) ^ 1, a.status, a.polls))
      return false;
    if (*c.abort_flag) return false;
    const int nk = min(g::ks, nks - i);
    unsigned char* st = c.smem + s * OZ_SLOT;
    mbar_expect_tx(&c.full[s], 2 * nk * g::nsl * OZ_BLK);
    for (int kk = 0; kk < nk; ++kk) {
      const size_t oa = ((size_t)mt * a.nK16 + ks0 + i + kk) * (OZ_BLK / 2);
      const size_t ob = ((size_t)nt * a.nK16 + ks0 + i + kk) * (OZ_BLK / 2);
#pragma unroll
      for (int sl = 0; sl < g::nsl; ++sl) {
        bulk_g2s(st + (kk * g::nsl + sl) * OZ_BLK, a.A + sl * sliceA + oa, OZ_BLK, &c.full[s]);
        bulk_g2s(st + ((g::ks + kk) * g::nsl + sl) * OZ_BLK, a.B + sl * sliceB + ob, OZ_BLK,
                 &c.full[s]);
      }
    }
    issued = q + 1;
  }
  return true;
}

// MMA issuer, one group: windows of g::win K steps; at a window's start the
// accumulators it takes (blocks 0 .. nd-1) must have been read by the
// epilogue; at its end each is committed to its accfull barrier.  used/par:
// per accumulator, used at least once / parity of its use count.
template <int G>
__device__ __forceinline__ bool oz_mma(const OzArgs& a, const OzCta& c, uint32_t idesc, int nks,
                                       int& q, uint32_t& used, uint32_t& par) {
  using g = OzG<G>;
  for (int w0 = 0; w0 < nks; w0 += g::win) {
    const int w1 = min(nks, w0 + g::win);
    int bb[3];
    uint32_t tb[3];
#pragma unroll
    for (int k = 0; k < g::nd; ++k) {
      bb[k] = k;
      tb[k] = c.tbase + (uint32_t)(bb[k] * 128);
      if ((used >> bb[k]) & 1) {
        if (!mbar_wait(&c.accempty[bb[k]], ((par >> bb[k]) & 1) ^ 1, a.status, a.polls))
          return false;
      }
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    for (int i = w0; i < w1; i += g::ks, ++q) {
      const int s = q % OZ_STAGES;
      if (!mbar_wait(&c.full[s], (q / OZ_STAGES) & 1, a.status, a.polls)) return false;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint64_t d0 = sdesc(su32(c.smem + s * OZ_SLOT));
      const int nk = min(g::ks, w1 - i);
#pragma unroll
      for (int kk = 0; kk < g::ks; ++kk) {
        if (kk < nk) {
          const uint32_t first_step = (i == w0 && kk == 0) ? 1u : 0u;
#pragma unroll
          for (int pp = 0; pp < g::np; ++pp) {
            const int k = g::acc(pp);
            const uint64_t da = d0 + (uint64_t)(((kk * g::nsl + g::ia(pp)) * OZ_BLK) >> 4);
            const uint64_t db =
                d0 + (uint64_t)((((g::ks + kk) * g::nsl + oz_jb<g>(pp)) * OZ_BLK) >> 4);
            const uint32_t accf = (pp == g::first(k)) ? (first_step ^ 1u) : 1u;
            mma_f16(tb[k], da, db, idesc, accf);
          }
        }
      }
      mma_commit(&c.empty[s]);  // frees the stage once these MMAs are done
    }
#pragma unroll
    for (int k = 0; k < g::nd; ++k) {
      mma_commit(&c.accfull[bb[k]]);
      used |= 1u << bb[k];
      par ^= 1u << bb[k];
    }
  }
  return true;
}

// Epilogue, one group: fold each closed accumulator (an exact integer sum
// times 2^(-7 d)) into the compensated pair (hi, lo): hi in registers, lo in
// the fourth tensor-memory block (columns 384-511).  The accumulator is
// released as soon as it is in registers.
template <int G>
__device__ __forceinline__ bool oz_fold(const OzArgs& a, const OzCta& c, uint32_t taddr, int nks,
                                        uint32_t& par, float* hi) {
  using g = OzG<G>;
  for (int w0 = 0; w0 < nks; w0 += g::win) {
#pragma unroll
    for (int k = 0; k < g::nd; ++k) {
      if (!mbar_wait(&c.accfull[k], (par >> k) & 1, a.status, a.polls)) return false;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // 2^(-7 d) as an FP32 bit pattern (d <= 8: exponent >= -56)
      const float sc = __uint_as_float((uint32_t)(127 - 7 * g::diag(k)) << 23);
      uint32_t v[OZ_ECOLS];
      tmem_ld16(taddr + k * 128, v);
      tmem_ld16(taddr + k * 128 + 16, v + 16);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(&c.accempty[k]);
      par ^= 1u << k;
#pragma unroll
      for (int h = 0; h < OZ_ECOLS; h += 16) {
        uint32_t l[16];
        tmem_ld16(taddr + 3 * 128 + h, l);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const float x = __uint_as_float(v[h + j]) * sc;
          const float y = hi[h + j];
          const float s = y + x;
          const float bbv = s - y;
          const float e = (y - (s - bbv)) + (x - bbv);
          hi[h + j] = s;
          l[j] = __float_as_uint(__uint_as_float(l[j]) + e);
        }
        tmem_st16(taddr + 3 * 128 + h, l);
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      }
    }
  }
  return true;
}

// x 2^e for |e| <= 2044 by two exact power-of-two products (no libm call)
__device__ __forceinline__ double oz_scale2(double x, int e) {
  const int e1 = e / 2, e2 = e - e1;
  return x * __longlong_as_double((long long)(1023 + e1) << 52) *
         __longlong_as_double((long long)(1023 + e2) << 52);
}

template <int MODE>
__global__ void __launch_bounds__(OZ_THREADS, 1) k_oz_gemm(OzArgs args) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  OzCta c;
  c.smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  c.full = (uint64_t*)(c.smem + OZ_STAGES * OZ_SLOT);
  c.empty = c.full + OZ_STAGES;
  c.accfull = c.empty + OZ_STAGES;
  c.accempty = c.accfull + OZ_NBUF;
  c.drain = c.accempty + OZ_NBUF;
  uint32_t* tmem_slot = (uint32_t*)(c.drain + 1);
  c.abort_flag = (volatile int*)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nt = blockIdx.x, mt = blockIdx.y, z = blockIdx.z;
  const int ks0 = z * args.k16_per_split;
  const int nks = *(volatile const int*)args.status ? 0
                                                    : min(args.k16_per_split, args.nK16 - ks0);
  const bool g3 = args.nsl >= 7;

  if (threadIdx.x == 0) {
    for (int s = 0; s < OZ_STAGES; ++s) {
      mbar_init(&c.full[s], 1);
      mbar_init(&c.empty[s], 1);
    }
    for (int b = 0; b < OZ_NBUF; ++b) {
      mbar_init(&c.accfull[b], 1);
      mbar_init(&c.accempty[b], OZ_EPI);
    }
    mbar_init(c.drain, 1);
    *c.abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     su32(tmem_slot)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  c.tbase = *tmem_slot;
  if (nks > 0) {
    if (warp == 0 && lane == 0) {
      // ---------------- producer
      int q = 0, issued = 0;
      bool ok = oz_produce<0>(args, c, mt, nt, ks0, nks, q, issued) &&
                oz_produce<1>(args, c, mt, nt, ks0, nks, q, issued) &&
                (!g3 || oz_produce<2>(args, c, mt, nt, ks0, nks, q, issued));
      if (!ok) {
        *c.abort_flag = 1;
        atomicExch(args.status, 1);
      }
      // no copy may still be landing in shared memory when the CTA retires
      for (int i = max(0, issued - OZ_STAGES); i < issued; ++i)
        if (!mbar_wait_drain(&c.full[i % OZ_STAGES], (i / OZ_STAGES) & 1)) {
          *c.abort_flag = 1;
          atomicExch(args.status, 1);
        }
    } else if (warp == 1 && lane == 0) {
      // ---------------- MMA issuer
      // the last N tile multiplies only its valid rows of B (rounded up to
      // the MMA's multiple of 16): no tensor work on padding rows
      const uint32_t idesc =
          idesc_f16_f32(OZ_M, min(OZ_N, (args.N - nt * OZ_N + 15) & ~15));
      int q = 0;
      uint32_t used = 0, par = 0;
      const bool ok = oz_mma<0>(args, c, idesc, nks, q, used, par) &&
                      oz_mma<1>(args, c, idesc, nks, q, used, par) &&
                      (!g3 || oz_mma<2>(args, c, idesc, nks, q, used, par));
      if (!ok) {
        *c.abort_flag = 1;
        atomicExch(args.status, 1);
      }
      // every MMA of this thread has completed before tensor memory is freed
      mma_commit(c.drain);
      if (!mbar_wait_drain(c.drain, 0)) {
        *c.abort_flag = 1;
        atomicExch(args.status, 1);
      }
    } else if (warp >= 2) {
      // ---------------- epilogue: warp w reads tensor-memory lane quarter
      // w & 3 and 32 of the 128 columns of each accumulator
      const int qd = warp & 3;
      const int cbase = ((warp - 2) >> 2) * OZ_ECOLS;
      const uint32_t taddr = c.tbase + ((uint32_t)(qd * 32) << 16) + (uint32_t)cbase;
      float hi[OZ_ECOLS];
#pragma unroll
      for (int j = 0; j < OZ_ECOLS; ++j) hi[j] = 0.f;
      {
        uint32_t zero[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) zero[j] = 0u;
        tmem_st16(taddr + 3 * 128, zero);
        tmem_st16(taddr + 3 * 128 + 16, zero);
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      }
      uint32_t par = 0;
      bool ok = oz_fold<0>(args, c, taddr, nks, par, hi) &&
                oz_fold<1>(args, c, taddr, nks, par, hi) &&
                (!g3 || oz_fold<2>(args, c, taddr, nks, par, hi));
      if (!ok) {
        *c.abort_flag = 1;
        atomicExch(args.status, 1);
      }
      // final write once the MMA thread's drain has completed
      if (ok && !mbar_wait_drain(c.drain, 0)) {
        *c.abort_flag = 1;
        atomicExch(args.status, 1);
        ok = false;
      }
      if (ok && !*c.abort_flag) {
        uint32_t lo[OZ_ECOLS];
        tmem_ld16(taddr + 3 * 128, lo);
        tmem_ld16(taddr + 3 * 128 + 16, lo + 16);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        const int m = mt * OZ_M + qd * 32 + lane;
        if (m < args.M) {
          const int ea = args.eA[m];
#pragma unroll
          for (int j = 0; j < OZ_ECOLS; ++j) {
            const int n = nt * OZ_N + cbase + j;
            if (n < args.N) {
              const double v = oz_scale2((double)hi[j] + (double)__uint_as_float(lo[j]),
                                         ea + args.eB[n]);
              if (MODE == OZ_OUT_PARTIAL)
                args.out[((size_t)z * args.N + n) * args.M + m] = v;
              else
                args.out[(size_t)n * 2 * args.ldo + m] = v;
            }
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(c.tbase), "r"(512));
}

// fnl[n][p] = (D_p/Omega) sum_z part[z][n][2p + c]; E_nl partials
__global__ void k_oz_fnl_reduce(const double* __restrict__ part, int nsplit, int M, int nst,
                                const double* __restrict__ wt, const double* __restrict__ occ,
                                double2* __restrict__ fnl, double* __restrict__ enl_part) {
  __shared__ double red[256];
  const int P = M / 2;
  const size_t total = (size_t)P * nst;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double e = 0.0;
  if (i < total) {
    const int n = (int)(i / P), p = (int)(i - (size_t)n * P);
    double re = 0.0, im = 0.0;
    for (int zz = 0; zz < nsplit; ++zz) {
      const double* pz = part + ((size_t)zz * nst + n) * M;
      re += pz[2 * p];
      im += pz[2 * p + 1];
    }
    const double fac = wt[p];
    e = (fac * (occ ? occ[n] : 0.0)) * (re * re + im * im);
    fnl[i] = make_double2(fac * re, fac * im);
  }
  red[threadIdx.x] = e;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0 && enl_part) enl_part[blockIdx.x] = red[0];
}

// ------------------------------------------------------------- host side
struct OzTables {
  int P = 0, ngw = 0, nsl = 0;
  int x1_RT = 0, x1_K16 = 0, x2_RT = 0, x2_K16 = 0;
  __half* X1 = nullptr;
  __half* X2 = nullptr;
  int* e1 = nullptr;   // per-row exponents of X1 (2P)
  int* e2 = nullptr;   // per-row exponents of X2 (2 ngw)
  unsigned long long* pmax = nullptr;  // per-projector maxima (P)
  unsigned long long* gmax = nullptr;  // per-G maxima (ngw)
  // per-H scratch
  __half* Y = nullptr;  size_t Y_bytes = 0;
  __half* F = nullptr;  size_t F_bytes = 0;
  int* eY = nullptr;    size_t eY_bytes = 0;
  int* eF = nullptr;    size_t eF_bytes = 0;
  unsigned long long* rmax = nullptr; size_t rmax_bytes = 0;
  double* part = nullptr; size_t part_bytes = 0;
  double2* fnl = nullptr; size_t fnl_bytes = 0;
  int* status = nullptr;
  int* h_status = nullptr;
  bool stale = false;
};

size_t slices_bytes(int nsl, int nRT, int nK16) { return (size_t)nsl * nRT * nK16 * OZ_BLK; }

void oz_free(OzTables* t) {
  if (!t) return;
  void* bufs[] = {t->X1, t->X2, t->e1, t->e2, t->pmax, t->gmax, t->Y, t->F, t->eY, t->eF,
                  t->rmax, t->part, t->fnl, t->status};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (t->h_status) cudaFreeHost(t->h_status);
  delete t;
}

qbg_status ensure_slices(__half** buf, size_t* cur, size_t need, cudaStream_t st) {
  const void* before = *buf;
  QBG_TRY_OZ(ensure((void**)buf, cur, need));
  if (*buf != before) QBG_CUDA(cudaMemsetAsync(*buf, 0, *cur, st));  // padding stays zero
  return QBG_OK;
}

int sm_count() {
  int sms = 152, dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

template <int MODE>
qbg_status oz_launch(qbg_plan* p, const OzArgs& a, int mt, int nt, int nsplit, cudaStream_t st) {
  if (mt > 65535 || nsplit > 65535) {
    set_error("FP64 tensor-core GEMM: %d row tiles exceed the grid limit", mt);
    return QBG_ERR_UNSUPPORTED;
  }
  QBG_CUDA(cudaFuncSetAttribute(k_oz_gemm<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                OZ_SMEM));
  k_oz_gemm<MODE><<<dim3(nt, mt, nsplit), OZ_THREADS, OZ_SMEM, st>>>(a);
  QBG_LAUNCHED(p);
  return QBG_OK;
}

}  // namespace

// Slices of the plan's projector table (rebuilt when the table changes;
// buffers of the same shape are reused).
qbg_status oz_build(qbg_plan* p, cudaStream_t st) {
  OzTables* t = (OzTables*)p->oz;
  const int nsl = p->oz_slices;
  if (t && (t->P != p->nproj || t->ngw != p->ngw || t->nsl != nsl)) {
    oz_release(p);
    t = nullptr;
  }
  if (p->nproj == 0 || p->ngw == 0) {
    oz_release(p);
    return QBG_OK;
  }
  if (!t) {
    t = new OzTables;
    p->oz = t;
    t->P = p->nproj;
    t->ngw = p->ngw;
    t->nsl = nsl;
    t->x1_RT = (2 * t->P + OZ_M - 1) / OZ_M;
    t->x1_K16 = (2 * t->ngw + 15) / 16;
    t->x2_RT = (2 * t->ngw + OZ_M - 1) / OZ_M;
    t->x2_K16 = (2 * t->P + 15) / 16;
    const size_t b1 = slices_bytes(nsl, t->x1_RT, t->x1_K16);
    const size_t b2 = slices_bytes(nsl, t->x2_RT, t->x2_K16);
    QBG_CUDA(cudaMalloc(&t->X1, b1));
    QBG_CUDA(cudaMalloc(&t->X2, b2));
    QBG_CUDA(cudaMemsetAsync(t->X1, 0, b1, st));
    QBG_CUDA(cudaMemsetAsync(t->X2, 0, b2, st));
    QBG_CUDA(cudaMalloc(&t->e1, sizeof(int) * 2 * t->P));
    QBG_CUDA(cudaMalloc(&t->e2, sizeof(int) * 2 * (size_t)t->ngw));
    QBG_CUDA(cudaMalloc(&t->pmax, sizeof(unsigned long long) * t->P));
    QBG_CUDA(cudaMalloc(&t->gmax, sizeof(unsigned long long) * t->ngw));
    QBG_CUDA(cudaMalloc(&t->status, sizeof(int)));
    QBG_CUDA(cudaMemsetAsync(t->status, 0, sizeof(int), st));
  }
  t->stale = false;
  QBG_CUDA(cudaMemsetAsync(t->pmax, 0, sizeof(unsigned long long) * t->P, st));
  k_oz_rowmax<<<dim3(std::min(32, (t->ngw + 255) / 256), t->P), 256, 0, st>>>(p->d_anl, t->ngw,
                                                                             t->ngw, t->pmax);
  QBG_LAUNCHED(p);
  k_oz_colmax<<<(t->ngw + 255) / 256, 256, 0, st>>>(p->d_anl, t->P, t->ngw, t->gmax);
  QBG_LAUNCHED(p);
  dim3 g((t->ngw + 255) / 256, t->P);
  k_oz_split_x1<<<g, 256, 0, st>>>(p->d_anl, t->P, t->ngw, t->pmax, nsl, t->X1, t->x1_RT,
                                   t->x1_K16, t->e1);
  QBG_LAUNCHED(p);
  k_oz_split_x2<<<g, 256, 0, st>>>(p->d_anl, t->P, t->ngw, t->gmax, nsl, t->X2, t->x2_RT,
                                   t->x2_K16, t->e2);
  QBG_LAUNCHED(p);
  return QBG_OK;
}

void oz_release(qbg_plan* p) {
  oz_free((OzTables*)p->oz);
  p->oz = nullptr;
}

void oz_invalidate(qbg_plan* p) {
  if (p->oz) ((OzTables*)p->oz)->stale = true;
}

// out[n][g] = sum_p anl[p][g] fnl[n][p] with fnl = D/Omega <anl|psi>, both
// GEMMs FP64-accurate on the tensor cores; psi and out FP64 [ld x nst];
// E_nl partial sums into enl_part when given.
qbg_status oz_nl_apply(qbg_plan* p, const double2* psi, int ld, double2* out, int nst,
                       const double* d_occ, double* enl_part, int* enl_blocks, cudaStream_t st) {
  OzTables* t = (OzTables*)p->oz;
  if (!t || t->stale) QBG_TRY_OZ(oz_build(p, st));
  t = (OzTables*)p->oz;
  *enl_blocks = 0;
  if (!t || nst == 0) return QBG_OK;
  const int P = t->P, ngw = t->ngw, nsl = t->nsl;
  const int nRT = (nst + OZ_N - 1) / OZ_N;
  const int polls = p->tc_polls >= 0 ? p->tc_polls : TC_SPIN;
  QBG_TRY_OZ(ensure_slices(&t->Y, &t->Y_bytes, slices_bytes(nsl, nRT, t->x1_K16), st));
  QBG_TRY_OZ(ensure_slices(&t->F, &t->F_bytes, slices_bytes(nsl, nRT, t->x2_K16), st));
  QBG_TRY_OZ(ensure((void**)&t->eY, &t->eY_bytes, sizeof(int) * nRT * OZ_N));
  QBG_TRY_OZ(ensure((void**)&t->eF, &t->eF_bytes, sizeof(int) * nRT * OZ_N));
  QBG_TRY_OZ(ensure((void**)&t->rmax, &t->rmax_bytes, sizeof(unsigned long long) * nst));
  QBG_TRY_OZ(ensure((void**)&t->fnl, &t->fnl_bytes, sizeof(double2) * (size_t)P * nst));
  {
    PhaseTimer pt(p, PH_MISC, st);
    QBG_CUDA(cudaMemsetAsync(t->rmax, 0, sizeof(unsigned long long) * nst, st));
    k_oz_rowmax<<<dim3(std::min(32, (ngw + 255) / 256), nst), 256, 0, st>>>(psi, ld, ngw,
                                                                          t->rmax);
    QBG_LAUNCHED(p);
    k_oz_split_rows<<<dim3((ngw + 1023) / 1024, nst), 256, 0, st>>>(psi, ld, ngw, t->rmax, nsl,
                                                                   t->Y, nRT, t->x1_K16, t->eY);
    QBG_LAUNCHED(p);
  }
  // GEMM1 split over K so that the CTAs (one per SM) fill their last wave
  const int sms = sm_count();
  const int tiles = t->x1_RT * nRT;
  int nsplit = 1;
  double best = 1e30;
  for (int ns = 1; ns <= 64 && ns <= t->x1_K16; ++ns) {
    const int waves = (tiles * ns + sms - 1) / sms;
    if (ns > 1 && waves > 8) break;
    const double cost = (double)waves / ns + 0.002 * ns;
    if (cost < best) {
      best = cost;
      nsplit = ns;
    }
  }
  const int ksp = (t->x1_K16 + nsplit - 1) / nsplit;
  nsplit = (t->x1_K16 + ksp - 1) / ksp;
  QBG_TRY_OZ(ensure((void**)&t->part, &t->part_bytes, sizeof(double) * nsplit * nst * 2 * P));
  OzArgs a1;
  a1.A = t->X1;
  a1.B = t->Y;
  a1.nRTa = t->x1_RT;
  a1.nRTb = nRT;
  a1.nK16 = t->x1_K16;
  a1.nsl = nsl;
  a1.M = 2 * P;
  a1.N = nst;
  a1.k16_per_split = ksp;
  a1.eA = t->e1;
  a1.eB = t->eY;
  a1.out = t->part;
  a1.ldo = 0;
  a1.status = t->status;
  a1.polls = polls;
  {
    PhaseTimer pt(p, PH_FNL_GEMM, st);
    QBG_TRY_OZ(oz_launch<OZ_OUT_PARTIAL>(p, a1, t->x1_RT, nRT, nsplit, st));
  }
  const size_t total = (size_t)P * nst;
  const int rb = (int)((total + 255) / 256);
  *enl_blocks = rb;
  {
    PhaseTimer pt(p, PH_FNL_REDUCE, st);
    k_oz_fnl_reduce<<<rb, 256, 0, st>>>(t->part, nsplit, 2 * P, nst, p->d_pwt, d_occ, t->fnl,
                                        enl_part);
    QBG_LAUNCHED(p);
    if (p->fnl_export)
      QBG_CUDA(cudaMemcpyAsync(p->fnl_export, t->fnl, sizeof(double2) * total,
                               cudaMemcpyDeviceToDevice, st));
    QBG_CUDA(cudaMemsetAsync(t->rmax, 0, sizeof(unsigned long long) * nst, st));
    k_oz_rowmax<<<dim3(std::min(32, (P + 255) / 256), nst), 256, 0, st>>>(t->fnl, P, P, t->rmax);
    QBG_LAUNCHED(p);
    k_oz_split_rows<<<dim3((P + 1023) / 1024, nst), 256, 0, st>>>(t->fnl, P, P, t->rmax, nsl,
                                                                 t->F, nRT, t->x2_K16, t->eF);
    QBG_LAUNCHED(p);
  }
  // GEMM2 writes the nonlocal part of H psi
  OzArgs a2;
  a2.A = t->X2;
  a2.B = t->F;
  a2.nRTa = t->x2_RT;
  a2.nRTb = nRT;
  a2.nK16 = t->x2_K16;
  a2.nsl = nsl;
  a2.M = 2 * ngw;
  a2.N = nst;
  a2.k16_per_split = t->x2_K16;
  a2.eA = t->e2;
  a2.eB = t->eF;
  a2.out = (double*)out;
  a2.ldo = ld;
  a2.status = t->status;
  a2.polls = polls;
  {
    PhaseTimer pt(p, PH_ENL_HPSI, st);
    QBG_TRY_OZ(oz_launch<OZ_OUT_HPSI>(p, a2, t->x2_RT, nRT, 1, st));
  }
  return QBG_OK;
}

// Reads the error word of the FP64 tensor-core GEMMs on the caller's stream.
qbg_status oz_check_status(qbg_plan* p, cudaStream_t st) {
  OzTables* t = (OzTables*)p->oz;
  if (!t) return QBG_OK;
  if (!t->h_status) QBG_CUDA(cudaMallocHost(&t->h_status, sizeof(int)));
  *t->h_status = 0;
  QBG_CUDA(cudaMemcpyAsync(t->h_status, t->status, sizeof(int), cudaMemcpyDeviceToHost, st));
  QBG_CUDA(cudaStreamSynchronize(st));
  if (*t->h_status) {
    set_error("FP64 tensor-core GEMM: a bounded wait expired (status %d)", *t->h_status);
    QBG_CUDA(cudaMemsetAsync(t->status, 0, sizeof(int), st));
    QBG_CUDA(cudaStreamSynchronize(st));
    return QBG_ERR_TIMEOUT;
  }
  return QBG_OK;
}

}  // namespace qbg
