// qbg_tc.cu -- projector GEMMs on the 5th-generation tensor cores (tcgen05).
//
// Mixed precision form of NonLocalPotential::energy (NonLocalPotential.cc:
// 2059-2170).  Both complex GEMMs are rewritten as real GEMMs D = A B^T with
// K-major operands:
//   GEMM1  D[2P x nst]    = X1[2P x 2ngw]  * Psi[nst x 2ngw]^T   -> fnl
//   GEMM2  D[2ngw x nst]  = X2[2ngw x 2P]  * Fnl[nst x 2P]^T     -> H psi (NL part)
// where Psi and Fnl are the interleaved (re,im) views of the wavefunctions
// and projections, and X1 (X2 = X1^T) interleaves anl so that one real dot
// product yields the real or imaginary part (X1[2p][2g]=re, [2p][2g+1]=im,
// [2p+1][2g]=-im, [2p+1][2g+1]=re).
//
// Precision: every operand row is scaled by a power of two and split into two
// FP16 pieces (hi = fp16(x), lo = fp16(x - hi): 22 significant bits).  Three
// products hi*hi + hi*lo + lo*hi run as kind::f16 MMAs (M=128, N=128, K=16)
// accumulating in FP32 in tensor memory.  Every 256 K-elements the chunk sum
// is folded into a compensated (hi, lo) FP32 pair that also lives in tensor
// memory, so the total carries ~FP64-class accumulation error and FP32-class
// operand error.
//
// Data movement: operands are pre-split into a tile-canonical layout in HBM
// (each 128x32 block of a piece is one contiguous 8 KB image of the shared-
// memory canonical K-major layout), so the producer warp moves them with 1-D
// bulk async copies (cp.async.bulk, completion on an mbarrier).
//
// Warp roles (192 threads): warp 0 producer, warp 1 MMA issuer, warps 2-5
// epilogue (tensor-memory lane quarters 2,3,0,1).  Every wait is bounded; a
// timeout sets an error word, the CTA drains and frees its tensor memory.
#include <algorithm>
#include <cstdint>
#include <cuda_fp16.h>
#include <vector>

#include "qbg_internal.h"
#include "qbg_tcgen05.cuh"

namespace qbg {

#define QBG_TRY_TC(x)             \
  do {                            \
    qbg_status s_ = (x);          \
    if (s_ != QBG_OK) return s_;  \
  } while (0)

constexpr int TC_M = 128;          // rows per tile (A)
constexpr int TC_N = 128;          // rows per tile (B) = MMA N
constexpr int TC_KS = 32;          // K elements per pipeline stage
#ifndef QBG_TC_STAGES
#define QBG_TC_STAGES 4
#endif
constexpr int TC_STAGES = QBG_TC_STAGES;
#ifndef QBG_TC_CHUNK
#define QBG_TC_CHUNK 8
#endif
constexpr int TC_CHUNK = QBG_TC_CHUNK;  // stages per tensor-memory chunk (K = 256)
constexpr int TC_BLOCK_BYTES = TC_M * TC_KS * 2;   // 8 KB per piece per stage
constexpr int TC_STAGE_BYTES = 4 * TC_BLOCK_BYTES; // A0 A1 B0 B1
constexpr int TC_THREADS = 576;    // producer, MMA issuer, 16 epilogue warps
constexpr int TC_NBUF = 4;         // tensor-memory chunk buffers (4 x 128 columns)
constexpr int TC_EPI = 512;        // epilogue threads
constexpr int TC_ECOLS = 32;       // columns per epilogue thread

// byte offset of element (r, k) inside one 128x32 block image
__host__ __device__ __forceinline__ int tc_canon(int r, int k) {
  const int kk = k >> 4, kl = k & 15;
  return kk * 4096 + (r >> 3) * 256 + (kl >> 3) * 128 + (r & 7) * 16 + (kl & 7) * 2;
}

// element offset (in halves) of (piece, row, k) in a tile-canonical array
// with nRT row tiles and nKS K stages
__host__ __device__ __forceinline__ size_t tc_index(int piece, int r, int k, int nRT, int nKS) {
  const size_t blk = ((size_t)piece * nRT + (r >> 7)) * nKS + (k >> 5);
  return blk * (TC_BLOCK_BYTES / 2) + (tc_canon(r & 127, k & 31) >> 1);
}

// --------------------------------------------------------------- splitting
__device__ __forceinline__ void split2(float x, __half& hi, __half& lo) {
  hi = __float2half_rn(x);
  lo = __float2half_rn(x - __half2float(hi));
}

// exponent e with |x| * 2^-e < 2^14 for all |x| <= amax (0 when amax == 0)
__device__ __forceinline__ int scale_exp(double amax) {
  if (!(amax > 0.0)) return 0;
  int e;
  frexp(amax, &e);  // amax = f * 2^e, f in [0.5, 1)
  return e - 14;
}

// x 2^-e rounded to FP32 from the FP64 bit pattern (no FP64 instruction:
// GB300 runs FP64 at 1/72 of FP32); the power of two is applied after the
// conversion for |e| < 100 (values that underflow FP32 then are below 2^-110
// of the row maximum, far below the 22 bits the two pieces keep)
__device__ __forceinline__ float f32_scaled(double x, int e) {
  if (e > -100 && e < 100) return f32_from_f64_rn(x) * __uint_as_float((uint32_t)(127 - e) << 23);
  return __double2float_rn(ldexp(x, -e));
}

// per-projector and per-G maxima of |re|,|im| of anl[p][g], compared as the
// integer bit patterns with the sign cleared (no FP64 instruction)
__global__ void k_anl_rowmax(const double2* __restrict__ anl, int nproj, int ngw,
                             double* __restrict__ pmax) {
  __shared__ unsigned long long red[256];
  const int p = blockIdx.x;
  const unsigned long long mask = 0x7FFFFFFFFFFFFFFFull;
  unsigned long long m = 0;
  for (int g = threadIdx.x; g < ngw; g += blockDim.x) {
    const double2 a = anl[(size_t)p * ngw + g];
    m = max(m, max((unsigned long long)__double_as_longlong(a.x) & mask,
                   (unsigned long long)__double_as_longlong(a.y) & mask));
  }
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = max(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) pmax[p] = __longlong_as_double((long long)red[0]);
}

__global__ void k_anl_colmax(const double2* __restrict__ anl, int nproj, int ngw,
                             double* __restrict__ gmax) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ngw) return;
  const unsigned long long mask = 0x7FFFFFFFFFFFFFFFull;
  unsigned long long m = 0;
  for (int p = 0; p < nproj; ++p) {
    const double2 a = anl[(size_t)p * ngw + g];
    m = max(m, max((unsigned long long)__double_as_longlong(a.x) & mask,
                   (unsigned long long)__double_as_longlong(a.y) & mask));
  }
  gmax[g] = __longlong_as_double((long long)m);
}

// X1 pieces: rows 2p+c, K = 2ngw; element values of the interleaved form
__global__ void k_split_x1(const double2* __restrict__ anl, int nproj, int ngw,
                           const double* __restrict__ pmax, __half* __restrict__ X1,
                           int nRT, int nKS, float* __restrict__ rscale) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int p = blockIdx.y;
  const int e = scale_exp(pmax[p]);
  if (g == 0) {
    rscale[2 * p] = ldexpf(1.f, e);
    rscale[2 * p + 1] = ldexpf(1.f, e);
  }
  if (g >= ngw) return;
  const double2 a = anl[(size_t)p * ngw + g];
  const float re = f32_scaled(a.x, e), im = f32_scaled(a.y, e);
  __half rh, rl, ih, il;
  split2(re, rh, rl);
  split2(im, ih, il);
  // (2p,2g) = re, (2p,2g+1) = im, (2p+1,2g) = -im, (2p+1,2g+1) = re
  *reinterpret_cast<__half2*>(X1 + tc_index(0, 2 * p, 2 * g, nRT, nKS)) = __halves2half2(rh, ih);
  *reinterpret_cast<__half2*>(X1 + tc_index(1, 2 * p, 2 * g, nRT, nKS)) = __halves2half2(rl, il);
  *reinterpret_cast<__half2*>(X1 + tc_index(0, 2 * p + 1, 2 * g, nRT, nKS)) =
      __halves2half2(__hneg(ih), rh);
  *reinterpret_cast<__half2*>(X1 + tc_index(1, 2 * p + 1, 2 * g, nRT, nKS)) =
      __halves2half2(__hneg(il), rl);
}

// X2 = X1^T pieces: rows m = 2g+c, K = 2P, scaled per G
__global__ void k_split_x2(const double2* __restrict__ anl, int nproj, int ngw,
                           const double* __restrict__ gmax, __half* __restrict__ X2,
                           int nRT, int nKS, float* __restrict__ rscale) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int p = blockIdx.y;
  if (g >= ngw) return;
  const int e = scale_exp(gmax[g]);
  if (p == 0) {
    rscale[2 * g] = ldexpf(1.f, e);
    rscale[2 * g + 1] = ldexpf(1.f, e);
  }
  const double2 a = anl[(size_t)p * ngw + g];
  const float re = f32_scaled(a.x, e), im = f32_scaled(a.y, e);
  __half rh, rl, ih, il;
  split2(re, rh, rl);
  split2(im, ih, il);
  // X2[2g][2p]=re, X2[2g][2p+1]=-im, X2[2g+1][2p]=im, X2[2g+1][2p+1]=re
  *reinterpret_cast<__half2*>(X2 + tc_index(0, 2 * g, 2 * p, nRT, nKS)) =
      __halves2half2(rh, __hneg(ih));
  *reinterpret_cast<__half2*>(X2 + tc_index(1, 2 * g, 2 * p, nRT, nKS)) =
      __halves2half2(rl, __hneg(il));
  *reinterpret_cast<__half2*>(X2 + tc_index(0, 2 * g + 1, 2 * p, nRT, nKS)) =
      __halves2half2(ih, rh);
  *reinterpret_cast<__half2*>(X2 + tc_index(1, 2 * g + 1, 2 * p, nRT, nKS)) =
      __halves2half2(il, rl);
}

// row maxima of |re|, |im| of x[n][0..ncols): blocks (chunk, row), the block
// maxima combined with an integer atomicMax on the bit patterns (for
// non-negative doubles the order of the bits is the order of the values);
// rmax must be zero on entry
__global__ void k_rowmax_c64(const double2* __restrict__ x, int ld, int ncols,
                             double* __restrict__ rmax) {
  // maxima of |x| compared as the integer bit patterns with the sign
  // cleared (no FP64 instruction)
  __shared__ unsigned long long red[256];
  const int n = blockIdx.y;
  const unsigned long long mask = 0x7FFFFFFFFFFFFFFFull;
  unsigned long long m = 0;
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ncols; g += gridDim.x * blockDim.x) {
    const double2 a = x[(size_t)n * ld + g];
    const unsigned long long u = (unsigned long long)__double_as_longlong(a.x) & mask;
    const unsigned long long w = (unsigned long long)__double_as_longlong(a.y) & mask;
    m = max(m, max(u, w));
  }
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = max(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicMax(reinterpret_cast<unsigned long long*>(rmax) + n, red[0]);
}

// pieces of the interleaved real view of x[n][g] (K = 2*ncols), scaled per
// row; 4 complex elements (8 consecutive K, one 16-byte run of the canonical
// layout per piece) per thread, so every store fills whole sectors
__global__ void k_split_rows4(const double2* __restrict__ x, int ld, int ncols,
                              const double* __restrict__ rmax, __half* __restrict__ Y,
                              int nRT, int nKS, float* __restrict__ rscale, int n0) {
  // row blockIdx.y of x becomes row n0 + blockIdx.y of the pieces
  const int g0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int n = n0 + (int)blockIdx.y;
  x += (size_t)blockIdx.y * ld;
  const int e = scale_exp(rmax[n]);
  if (g0 == 0) rscale[n] = ldexpf(1.f, e);
  if (g0 >= ncols) return;
  // the split works on x 2^-e rounded to FP32 (24 bits, more than the 22 the
  // two pieces keep): one FP64-pipe conversion per value instead of the
  // FP64 scaling and residual, as GB300 runs FP64 at 1/72 of FP32.  For
  // |e| <= 100 the power of two is applied after the conversion (values
  // that underflow FP32 are below 2^-110 of the row maximum).
  const bool fscale = e > -100 && e < 100;
  const float sf = fscale ? ldexpf(1.f, -e) : 1.f;
  const double sd = ldexp(1.0, -e);
  __align__(16) __half hi[8], lo[8];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int g = g0 + j;
    const double2 a = g < ncols ? x[g] : make_double2(0.0, 0.0);
    const float xr = fscale ? f32_from_f64_rn(a.x) * sf : __double2float_rn(a.x * sd);
    const float xi = fscale ? f32_from_f64_rn(a.y) * sf : __double2float_rn(a.y * sd);
    split2(xr, hi[2 * j], lo[2 * j]);
    split2(xi, hi[2 * j + 1], lo[2 * j + 1]);
  }
  *reinterpret_cast<uint4*>(Y + tc_index(0, n, 2 * g0, nRT, nKS)) = *reinterpret_cast<uint4*>(hi);
  *reinterpret_cast<uint4*>(Y + tc_index(1, n, 2 * g0, nRT, nKS)) = *reinterpret_cast<uint4*>(lo);
}

// epilogue modes
enum { TC_OUT_PARTIAL = 0, TC_OUT_HPSI = 1 };

struct TcArgs {
  const __half* A;  // tile-canonical pieces, nRTa row tiles x nKS stages
  const __half* B;  // tile-canonical pieces, nRTb row tiles x nKS stages
  int nRTa, nRTb, nKS;
  int M, N;         // valid rows of A / B
  int ks_per_split; // K stages handled by one CTA (blockIdx.z)
  const float* sA;  // per-row scales of A (length M)
  const float* sB;  // per-row scales of B (length N)
  double* out;      // PARTIAL: [split][N][M] doubles; HPSI: complex out, real view
  int ldo;          // HPSI: leading dimension of out in complex elements
  int* status;      // error word (1 = a bounded wait expired)
  int polls;        // poll limit of the pipeline waits (the drains always use TC_SPIN)
};

template <int MODE>
__global__ void __launch_bounds__(TC_THREADS, 1) k_tc_gemm(TcArgs args) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1 KB alignment of the stage ring
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + TC_STAGES * TC_STAGE_BYTES);
  uint64_t* empty = full + TC_STAGES;
  uint64_t* accfull = empty + TC_STAGES;
  uint64_t* accempty = accfull + TC_NBUF;
  uint64_t* drain = accempty + TC_NBUF;
  uint32_t* tmem_slot = (uint32_t*)(drain + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // the N tiles of one M tile are adjacent in launch order, so the A block
  // (the large projector operand) is fetched from HBM once and re-read from L2
  const int nt = blockIdx.x, mt = blockIdx.y, z = blockIdx.z;
  const int ks0 = z * args.ks_per_split;
  // a CTA that starts after another one failed does no work
  const int nks = *(volatile const int*)args.status ? 0 : min(args.ks_per_split, args.nKS - ks0);
  const int nchunks = (nks + TC_CHUNK - 1) / TC_CHUNK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < TC_NBUF; ++b) {
      mbar_init(&accfull[b], 1);
      mbar_init(&accempty[b], TC_EPI);
    }
    mbar_init(drain, 1);
    *abort_flag = 0;
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
  const uint32_t tbase = *tmem_slot;
  // tensor memory columns: four chunk buffers of 128 columns; the running
  // sums live in the epilogue threads' registers
  if (nks > 0) {
    if (warp == 0 && lane == 0) {
      // ---------------- producer
      const size_t pieceA = (size_t)args.nRTa * args.nKS * (TC_BLOCK_BYTES / 2);
      const size_t pieceB = (size_t)args.nRTb * args.nKS * (TC_BLOCK_BYTES / 2);
      int issued = 0;
      for (int i = 0; i < nks; ++i) {
        const int s = i % TC_STAGES;
        const uint32_t par = ((i / TC_STAGES) & 1) ^ 1;
        if (i >= TC_STAGES && !mbar_wait(&empty[s], par, args.status, args.polls)) {
          *abort_flag = 1;
          atomicExch(args.status, 1);
          break;
        }
        if (*abort_flag) break;
        unsigned char* st = smem + s * TC_STAGE_BYTES;
        mbar_expect_tx(&full[s], TC_STAGE_BYTES);
        const size_t oa = ((size_t)mt * args.nKS + ks0 + i) * (TC_BLOCK_BYTES / 2);
        const size_t ob = ((size_t)nt * args.nKS + ks0 + i) * (TC_BLOCK_BYTES / 2);
        bulk_g2s(st, args.A + oa, TC_BLOCK_BYTES, &full[s]);
        bulk_g2s(st + TC_BLOCK_BYTES, args.A + pieceA + oa, TC_BLOCK_BYTES, &full[s]);
        bulk_g2s(st + 2 * TC_BLOCK_BYTES, args.B + ob, TC_BLOCK_BYTES, &full[s]);
        bulk_g2s(st + 3 * TC_BLOCK_BYTES, args.B + pieceB + ob, TC_BLOCK_BYTES, &full[s]);
        issued = i + 1;
      }
      // no copy may still be landing in shared memory when the CTA retires
      for (int i = max(0, issued - TC_STAGES); i < issued; ++i)
        if (!mbar_wait_drain(&full[i % TC_STAGES], (i / TC_STAGES) & 1)) {
          *abort_flag = 1;
          atomicExch(args.status, 1);
        }
    } else if (warp == 1 && lane == 0) {
      // ---------------- MMA issuer
      // the last N tile multiplies only its valid rows of B (rounded up to
      // the MMA's multiple of 16): no tensor work on padding rows
      const uint32_t idesc =
          idesc_f16_f32(TC_M, min(TC_N, (args.N - nt * TC_N + 15) & ~15));
      int i = 0;
      for (int c = 0; c < nchunks && !*abort_flag; ++c) {
        const int b = c % TC_NBUF;
        if (c >= TC_NBUF &&
            !mbar_wait(&accempty[b], ((c / TC_NBUF) - 1) & 1, args.status, args.polls)) {
          *abort_flag = 1;
          atomicExch(args.status, 1);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t dcol = tbase + (uint32_t)(b * 128);
        const int iend = min(nks, (c + 1) * TC_CHUNK);
        bool first = true;
        for (; i < iend; ++i) {
          const int s = i % TC_STAGES;
          if (!mbar_wait(&full[s], (i / TC_STAGES) & 1, args.status, args.polls)) {
            *abort_flag = 1;
            atomicExch(args.status, 1);
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t st = su32(smem + s * TC_STAGE_BYTES);
#pragma unroll
          for (int kk = 0; kk < 2; ++kk) {
            const uint64_t a0 = sdesc(st + kk * 4096);
            const uint64_t a1 = sdesc(st + TC_BLOCK_BYTES + kk * 4096);
            const uint64_t b0 = sdesc(st + 2 * TC_BLOCK_BYTES + kk * 4096);
            const uint64_t b1 = sdesc(st + 3 * TC_BLOCK_BYTES + kk * 4096);
            mma_f16(dcol, a0, b0, idesc, first ? 0u : 1u);
            first = false;
            mma_f16(dcol, a0, b1, idesc, 1u);
            mma_f16(dcol, a1, b0, idesc, 1u);
          }
          mma_commit(&empty[s]);  // frees the stage once these MMAs are done
        }
        if (*abort_flag) break;  // nobody folds this chunk; the drain below tracks its MMAs
        mma_commit(&accfull[b]);
      }
      // every MMA of this thread has completed before tensor memory is freed
      mma_commit(drain);
      if (!mbar_wait_drain(drain, 0)) {
        *abort_flag = 1;
        atomicExch(args.status, 1);
      }
    } else if (warp >= 2) {
      // ---------------- epilogue: fold each chunk into compensated (hi, lo)
      // sums held in registers.  Warp w reads tensor-memory lane quarter
      // w & 3 (rows) and column block (w - 2) >> 2 (32 of the 128 columns).
      const int q = warp & 3;
      const int cbase = ((warp - 2) >> 2) * TC_ECOLS;
      const uint32_t lane_off = (uint32_t)(q * 32) << 16;
      float hi[TC_ECOLS], lo[TC_ECOLS];
#pragma unroll
      for (int j = 0; j < TC_ECOLS; ++j) {
        hi[j] = 0.f;
        lo[j] = 0.f;
      }
      bool ok = true;
      for (int c = 0; c < nchunks; ++c) {
        const int b = c % TC_NBUF;
        if (!mbar_wait(&accfull[b], (c / TC_NBUF) & 1, args.status, args.polls)) {
          *abort_flag = 1;
          atomicExch(args.status, 1);
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
        for (int cb = 0; cb < TC_ECOLS; cb += 32) {
          uint32_t p[32];
          tmem_ld32(tbase + lane_off + b * 128 + cbase + cb, p);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const float x = __uint_as_float(p[j]);
            const float a = hi[cb + j];
            const float s = a + x;
            const float bb = s - a;
            const float e = (a - (s - bb)) + (x - bb);
            hi[cb + j] = s;
            lo[cb + j] += e;
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        mbar_arrive(&accempty[b]);
      }
      // final write from the registers, once the MMA thread's drain has
      // completed (every MMA of the tile is done)
      if (ok && !mbar_wait_drain(drain, 0)) {
        *abort_flag = 1;
        atomicExch(args.status, 1);
        ok = false;
      }
      if (ok && !*abort_flag) {
        const int m = mt * TC_M + q * 32 + lane;
        if (m < args.M) {
          const float sa = args.sA[m];
#pragma unroll
          for (int j = 0; j < TC_ECOLS; ++j) {
            const int n = nt * TC_N + cbase + j;
            if (n < args.N) {
              // sa * sB is a power of two: scaling the (hi, lo) pair in FP32
              // is exact, and the FP64 result then costs one FP64 add
              const float sc = sa * args.sB[n];
              const double v = f64_from_f32(hi[j] * sc) + f64_from_f32(lo[j] * sc);
              if (MODE == TC_OUT_PARTIAL)
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
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(512));
}

// ---------------------------------------------------------- reduce + split
// fnl[n][p] = (D_p/Omega) * sum_z part[z][n][2p + c]; E_nl partials; the
// per-state max |fnl| for the next split
__global__ void k_tc_fnl_reduce(const double* __restrict__ part, int nsplit, int M, int nst,
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
struct TcTables {
  int P = 0, ngw = 0;
  int x1_RT = 0, x1_KS = 0, x2_RT = 0, x2_KS = 0;
  __half* X1 = nullptr;
  __half* X2 = nullptr;
  float* s1 = nullptr;  // per-row scales of X1 (2P)
  float* s2 = nullptr;  // per-row scales of X2 (2ngw)
  // per-H scratch
  __half* Y = nullptr;  size_t Y_bytes = 0;
  __half* F = nullptr;  size_t F_bytes = 0;
  float* sY = nullptr;  size_t sY_bytes = 0;
  float* sF = nullptr;  size_t sF_bytes = 0;
  double* rmax = nullptr; size_t rmax_bytes = 0;
  double* part = nullptr; size_t part_bytes = 0;
  double2* fnl = nullptr; size_t fnl_bytes = 0;
  int* status = nullptr;
  int* h_status = nullptr; // pinned host copy of the error word
  double* pmax = nullptr;  // per-projector maxima of the table (P)
  double* gmax = nullptr;  // per-G maxima (ngw)
  bool stale = false;      // the table changed: re-split before the next use
};

static size_t pieces_bytes(int nRT, int nKS) { return 2ull * nRT * nKS * TC_BLOCK_BYTES; }

static void tc_free(TcTables* t) {
  if (!t) return;
  void* bufs[] = {t->X1, t->X2, t->s1, t->s2, t->Y, t->F, t->sY, t->sF, t->rmax, t->part, t->fnl,
                  t->status, t->pmax, t->gmax};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (t->h_status) cudaFreeHost(t->h_status);
  delete t;
}

void tc_release(qbg_plan* p) {
  tc_free((TcTables*)p->tc);
  p->tc = nullptr;
}

void tc_invalidate(qbg_plan* p) {
  if (p->tc) ((TcTables*)p->tc)->stale = true;
}

// Split the plan's table into the FP16 pieces; the buffers of a previous
// table of the same shape are reused (their zero padding stays valid).
qbg_status tc_build(qbg_plan* p, cudaStream_t st) {
  TcTables* t = (TcTables*)p->tc;
  if (t && (t->P != p->nproj || t->ngw != p->ngw)) {
    tc_release(p);
    t = nullptr;
  }
  if (p->nproj == 0 || p->ngw == 0) {
    tc_release(p);
    return QBG_OK;
  }
  if (!t) {
    t = new TcTables;
    p->tc = t;
    t->P = p->nproj;
    t->ngw = p->ngw;
    t->x1_RT = (2 * t->P + TC_M - 1) / TC_M;
    t->x1_KS = (2 * t->ngw + TC_KS - 1) / TC_KS;
    t->x2_RT = (2 * t->ngw + TC_M - 1) / TC_M;
    t->x2_KS = (2 * t->P + TC_KS - 1) / TC_KS;
    const size_t b1 = pieces_bytes(t->x1_RT, t->x1_KS), b2 = pieces_bytes(t->x2_RT, t->x2_KS);
    QBG_CUDA(cudaMalloc(&t->X1, b1));
    QBG_CUDA(cudaMalloc(&t->X2, b2));
    QBG_CUDA(cudaMemsetAsync(t->X1, 0, b1, st));
    QBG_CUDA(cudaMemsetAsync(t->X2, 0, b2, st));
    QBG_CUDA(cudaMalloc(&t->s1, sizeof(float) * 2 * t->P));
    QBG_CUDA(cudaMalloc(&t->s2, sizeof(float) * 2 * (size_t)t->ngw));
    QBG_CUDA(cudaMalloc(&t->status, sizeof(int)));
    QBG_CUDA(cudaMalloc(&t->pmax, sizeof(double) * t->P));
    QBG_CUDA(cudaMalloc(&t->gmax, sizeof(double) * t->ngw));
  }
  t->stale = false;
  QBG_CUDA(cudaMemsetAsync(t->status, 0, sizeof(int), st));
  k_anl_rowmax<<<t->P, 256, 0, st>>>(p->d_anl, t->P, t->ngw, t->pmax);
  QBG_LAUNCHED(p);
  k_anl_colmax<<<(t->ngw + 255) / 256, 256, 0, st>>>(p->d_anl, t->P, t->ngw, t->gmax);
  QBG_LAUNCHED(p);
  dim3 g((t->ngw + 255) / 256, t->P);
  k_split_x1<<<g, 256, 0, st>>>(p->d_anl, t->P, t->ngw, t->pmax, t->X1, t->x1_RT, t->x1_KS,
                                t->s1);
  QBG_LAUNCHED(p);
  k_split_x2<<<g, 256, 0, st>>>(p->d_anl, t->P, t->ngw, t->gmax, t->X2, t->x2_RT, t->x2_KS,
                                t->s2);
  QBG_LAUNCHED(p);
  return QBG_OK;
}

static qbg_status tc_launch(qbg_plan* p, int mode, const TcArgs& a, int mt, int nt, int nsplit,
                            cudaStream_t st) {
  if (mt > 65535 || nsplit > 65535) {
    set_error("tensor-core GEMM: %d row tiles exceed the grid limit", mt);
    return QBG_ERR_UNSUPPORTED;
  }
  const size_t smem = TC_STAGES * TC_STAGE_BYTES + 1024 + 256;
  if (mode == TC_OUT_PARTIAL) {
    QBG_CUDA(cudaFuncSetAttribute(k_tc_gemm<TC_OUT_PARTIAL>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_tc_gemm<TC_OUT_PARTIAL><<<dim3(nt, mt, nsplit), TC_THREADS, smem, st>>>(a);
  } else {
    QBG_CUDA(cudaFuncSetAttribute(k_tc_gemm<TC_OUT_HPSI>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_tc_gemm<TC_OUT_HPSI><<<dim3(nt, mt, nsplit), TC_THREADS, smem, st>>>(a);
  }
  QBG_LAUNCHED(p);
  return QBG_OK;
}

// Grows a piece array; a new allocation is cleared (its padding rows must
// stay zero).
static qbg_status ensure_pieces(__half** buf, size_t* cur, size_t need, cudaStream_t st) {
  const void* before = *buf;
  QBG_TRY_TC(ensure((void**)buf, cur, need));
  if (*buf != before) QBG_CUDA(cudaMemsetAsync(*buf, 0, *cur, st));
  return QBG_OK;
}

// GEMM1 of a projector table X1 (scales s1; x1_RT x x1_KS pieces of the
// plan's layout) with the nvec blocks of nst vectors xs[k] stacked as one
// operand of nvec * nst rows: split them into t->Y, leave the split-K partial
// sums in t->part ([nsplit][nvec * nst][2P]) and return nsplit.
static qbg_status tc_gemm1(qbg_plan* p, TcTables* t, const __half* X1, const float* s1,
                           const double2* const* xs, int nvec, int ld, int nst,
                           int* nsplit_out, cudaStream_t st) {
  const int P = t->P, ngw = t->ngw;
  const int nrows = nvec * nst;
  const int nRT = (nrows + TC_N - 1) / TC_N;
  QBG_TRY_TC(ensure_pieces(&t->Y, &t->Y_bytes, pieces_bytes(nRT, t->x1_KS), st));
  QBG_TRY_TC(ensure((void**)&t->sY, &t->sY_bytes, sizeof(float) * nRT * TC_N));
  QBG_TRY_TC(ensure((void**)&t->rmax, &t->rmax_bytes, sizeof(double) * nRT * TC_N));
  {
    PhaseTimer pt(p, PH_MISC, st);
    QBG_CUDA(cudaMemsetAsync(t->rmax, 0, sizeof(double) * nrows, st));
    for (int k = 0; k < nvec; ++k) {
      k_rowmax_c64<<<dim3(std::min(32, (ngw + 255) / 256), nst), 256, 0, st>>>(
          xs[k], ld, ngw, t->rmax + (size_t)k * nst);
      QBG_LAUNCHED(p);
      k_split_rows4<<<dim3((ngw + 1023) / 1024, nst), 256, 0, st>>>(
          xs[k], ld, ngw, t->rmax, t->Y, nRT, t->x1_KS, t->sY, k * nst);
      QBG_LAUNCHED(p);
    }
  }
  const int nst_all = nrows;
  const int mt1 = t->x1_RT;
  // split K so that the CTAs (one per SM) fill their last wave: the time is
  // ~ waves / nsplit, waves = ceil(tiles * nsplit / SMs); at least ~3 waves
  int sms = 152;
  {
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess)
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  }
  const int tiles = mt1 * nRT;
  int nsplit = 1;
  double best = 1e30;
  for (int ns = 1; ns <= 64 && ns <= t->x1_KS; ++ns) {
    const int waves = (tiles * ns + sms - 1) / sms;
    if (ns > 1 && waves > 8) break;
    const double cost = (double)waves / ns + 0.002 * ns;  // small cost per extra partial
    if (cost < best) {
      best = cost;
      nsplit = ns;
    }
  }
  const int ksp = (t->x1_KS + nsplit - 1) / nsplit;
  nsplit = (t->x1_KS + ksp - 1) / ksp;
  QBG_TRY_TC(ensure((void**)&t->part, &t->part_bytes, sizeof(double) * nsplit * nst_all * 2 * P));
  TcArgs a1;
  a1.A = X1;
  a1.B = t->Y;
  a1.nRTa = t->x1_RT;
  a1.nRTb = nRT;
  a1.nKS = t->x1_KS;
  a1.M = 2 * P;
  a1.N = nst_all;
  a1.ks_per_split = ksp;
  a1.sA = s1;
  a1.sB = t->sY;
  a1.out = t->part;
  a1.ldo = 0;
  a1.status = t->status;
  a1.polls = p->tc_polls >= 0 ? p->tc_polls : TC_SPIN;
  {
    PhaseTimer pt(p, PH_FNL_GEMM, st);
    QBG_TRY_TC(tc_launch(p, TC_OUT_PARTIAL, a1, mt1, nRT, nsplit, st));
  }
  *nsplit_out = nsplit;
  return QBG_OK;
}

// out[n][g] = sum_p anl[p][g] fnl[n][p] with fnl = D/Omega <anl|psi>; psi and
// out are FP64 [ld x nst]; enl partial sums into enl_part when given.
qbg_status tc_nl_apply(qbg_plan* p, const double2* psi, int ld, double2* out, int nst,
                       const double* d_occ, double* enl_part, int* enl_blocks,
                       cudaStream_t st) {
  TcTables* t = (TcTables*)p->tc;
  if (!t || t->stale) QBG_TRY_TC(tc_build(p, st));
  t = (TcTables*)p->tc;
  if (!t) return QBG_OK;
  const int P = t->P, ngw = t->ngw;
  const int nRT = (nst + TC_N - 1) / TC_N;
  QBG_TRY_TC(ensure_pieces(&t->F, &t->F_bytes, pieces_bytes(nRT, t->x2_KS), st));
  QBG_TRY_TC(ensure((void**)&t->sF, &t->sF_bytes, sizeof(float) * nRT * TC_N));
  QBG_TRY_TC(ensure((void**)&t->fnl, &t->fnl_bytes, sizeof(double2) * (size_t)P * nst));
  int nsplit = 1;
  QBG_TRY_TC(tc_gemm1(p, t, t->X1, t->s1, &psi, 1, ld, nst, &nsplit, st));
  const size_t total = (size_t)P * nst;
  const int rb = (int)((total + 255) / 256);
  *enl_blocks = rb;
  {
    PhaseTimer pt(p, PH_FNL_REDUCE, st);
    k_tc_fnl_reduce<<<rb, 256, 0, st>>>(t->part, nsplit, 2 * P, nst, p->d_pwt, d_occ, t->fnl,
                                        enl_part);
    QBG_LAUNCHED(p);
    if (p->fnl_export)
      QBG_CUDA(cudaMemcpyAsync(p->fnl_export, t->fnl, sizeof(double2) * total,
                               cudaMemcpyDeviceToDevice, st));
    QBG_CUDA(cudaMemsetAsync(t->rmax, 0, sizeof(double) * nst, st));
    k_rowmax_c64<<<dim3(std::min(32, (P + 255) / 256), nst), 256, 0, st>>>(t->fnl, P, P,
                                                                         t->rmax);
    QBG_LAUNCHED(p);
    k_split_rows4<<<dim3((P + 1023) / 1024, nst), 256, 0, st>>>(t->fnl, P, P, t->rmax, t->F,
                                                               nRT, t->x2_KS, t->sF, 0);
    QBG_LAUNCHED(p);
  }
  // GEMM2 writes the NL part of H psi
  TcArgs a2;
  a2.A = t->X2;
  a2.B = t->F;
  a2.nRTa = t->x2_RT;
  a2.nRTb = nRT;
  a2.nKS = t->x2_KS;
  a2.M = 2 * ngw;
  a2.N = nst;
  a2.ks_per_split = t->x2_KS;
  a2.sA = t->s2;
  a2.sB = t->sF;
  a2.out = (double*)out;
  a2.ldo = ld;
  a2.status = t->status;
  a2.polls = p->tc_polls >= 0 ? p->tc_polls : TC_SPIN;
  {
    PhaseTimer pt(p, PH_ENL_HPSI, st);
    QBG_TRY_TC(tc_launch(p, TC_OUT_HPSI, a2, t->x2_RT, nRT, 1, st));
  }
  return QBG_OK;
}

// ------------------------------------------- projections on other tables
// A second projector table (the derivative tables of the adjoint) in the
// same FP16 piece layout as the plan's GEMM1 operand.
struct TcProj {
  int P = 0, ngw = 0;
  __half* X1 = nullptr;
  float* s1 = nullptr;
  double* pmax = nullptr;
};

// f[n][p] = sum_z (part[z][n][2p], part[z][n][2p+1])
__global__ void k_tc_proj_sum(const double* __restrict__ part, int nsplit, int P, int nst,
                              double2* __restrict__ f) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)P * nst) return;
  const int n = (int)(i / P), q = (int)(i - (size_t)n * P);
  double re = 0.0, im = 0.0;
  for (int z = 0; z < nsplit; ++z) {
    const double* pz = part + ((size_t)z * nst + n) * 2 * P;
    re += pz[2 * q];
    im += pz[2 * q + 1];
  }
  f[i] = make_double2(re, im);
}

void tc_proj_free(void* h) {
  TcProj* q = (TcProj*)h;
  if (!q) return;
  if (q->X1) cudaFree(q->X1);
  if (q->s1) cudaFree(q->s1);
  if (q->pmax) cudaFree(q->pmax);
  delete q;
}

// Pieces of table (the plan's shape) into *proj, reusing its buffers when
// the shape is unchanged.
qbg_status tc_proj_build(qbg_plan* p, const double2* table, void** proj, cudaStream_t st) {
  TcTables* t = (TcTables*)p->tc;
  if (!t || t->stale) QBG_TRY_TC(tc_build(p, st));
  t = (TcTables*)p->tc;
  if (!t) return QBG_OK;
  TcProj* q = (TcProj*)*proj;
  if (q && (q->P != t->P || q->ngw != t->ngw)) {
    tc_proj_free(q);
    q = nullptr;
    *proj = nullptr;
  }
  if (!q) {
    q = new TcProj;
    *proj = q;
    q->P = t->P;
    q->ngw = t->ngw;
    const size_t b1 = pieces_bytes(t->x1_RT, t->x1_KS);
    QBG_CUDA(cudaMalloc(&q->X1, b1));
    QBG_CUDA(cudaMalloc(&q->s1, sizeof(float) * 2 * t->P));
    QBG_CUDA(cudaMalloc(&q->pmax, sizeof(double) * t->P));
    QBG_CUDA(cudaMemsetAsync(q->X1, 0, b1, st));
  }
  k_anl_rowmax<<<t->P, 256, 0, st>>>(table, t->P, t->ngw, q->pmax);
  QBG_LAUNCHED(p);
  dim3 g((t->ngw + 255) / 256, t->P);
  k_split_x1<<<g, 256, 0, st>>>(table, t->P, t->ngw, q->pmax, q->X1, t->x1_RT, t->x1_KS, q->s1);
  QBG_LAUNCHED(p);
  return QBG_OK;
}

// f[n][p] = sum_g conj(table[p][g]) x[n][g] on the tensor cores (no
// weights); proj == nullptr projects on the plan's own table.
qbg_status tc_project(qbg_plan* p, const void* proj, const double2* x, int ld, int nst,
                      double2* f, cudaStream_t st) {
  return tc_project_multi(p, proj, &x, 1, ld, nst, f, st);
}

// nvec blocks in one GEMM (the stacked rows fill the N tiles): f holds the
// nvec [nst][P] results one after the other
qbg_status tc_project_multi(qbg_plan* p, const void* proj, const double2* const* xs, int nvec,
                            int ld, int nst, double2* f, cudaStream_t st) {
  TcTables* t = (TcTables*)p->tc;
  if (!t || t->stale) QBG_TRY_TC(tc_build(p, st));
  t = (TcTables*)p->tc;
  if (!t || nst == 0 || nvec == 0) return QBG_OK;
  const TcProj* q = (const TcProj*)proj;
  int nsplit = 1;
  QBG_TRY_TC(tc_gemm1(p, t, q ? q->X1 : t->X1, q ? q->s1 : t->s1, xs, nvec, ld, nst, &nsplit, st));
  const int nrows = nvec * nst;
  const size_t total = (size_t)t->P * nrows;
  k_tc_proj_sum<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(t->part, nsplit, t->P, nrows, f);
  QBG_LAUNCHED(p);
  return QBG_OK;
}

// Diagnostic: one thread waits on an mbarrier that nothing completes, with
// `polls` polls; the wait must give up and report through the status word,
// leaving the context usable (the same bounded wait the GEMM's roles use).
__global__ void k_wait_selftest(int polls, int* status) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (!mbar_wait(&bar, 0, status, polls)) atomicExch(status, 1);
  }
}

// Reads the error word on the caller's stream (ordered after the launches
// it covers) into pinned host memory and synchronises that stream; a raised
// word is cleared on the same stream and reported as QBG_ERR_TIMEOUT.
qbg_status tc_check_status(qbg_plan* p, cudaStream_t st) {
  if (p->oz) {
    const qbg_status s = oz_check_status(p, st);
    if (s != QBG_OK) return s;
  }
  TcTables* t = (TcTables*)p->tc;
  if (!t) return QBG_OK;
  if (!t->h_status) QBG_CUDA(cudaMallocHost(&t->h_status, sizeof(int)));
  *t->h_status = 0;
  QBG_CUDA(cudaMemcpyAsync(t->h_status, t->status, sizeof(int), cudaMemcpyDeviceToHost, st));
  QBG_CUDA(cudaStreamSynchronize(st));
  const int s = *t->h_status;
  if (s) {
    set_error("tensor-core GEMM: a bounded wait expired (status %d)", s);
    QBG_CUDA(cudaMemsetAsync(t->status, 0, sizeof(int), st));
    QBG_CUDA(cudaStreamSynchronize(st));
    return QBG_ERR_TIMEOUT;
  }
  return QBG_OK;
}

}  // namespace qbg

extern "C" qbg_status qbg_selftest_wait_timeout(int polls) {
  using namespace qbg;
  if (polls < 1 || polls > (1 << 20)) {
    set_error("qbg_selftest_wait_timeout: polls must be in [1, 2^20]");
    return QBG_ERR_INVALID;
  }
  int* d = nullptr;
  QBG_CUDA(cudaMalloc(&d, sizeof(int)));
  cudaMemset(d, 0, sizeof(int));
  k_wait_selftest<<<1, 32>>>(polls, d);
  cudaError_t e = cudaGetLastError();
  int h = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_status(e, "qbg_selftest_wait_timeout");
  if (h) {
    set_error("bounded wait expired after %d polls (self-test)", polls);
    return QBG_ERR_TIMEOUT;
  }
  return QBG_OK;
}
