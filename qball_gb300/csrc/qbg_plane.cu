// qbg_plane.cu -- whole-plane fused x/y transforms of 120 x 120 planes.
//
// One CTA holds the complete (x, y) plane of one (z, state) pair in shared
// memory (120 rows of 121 elements: 232 320 bytes of 16-byte complex values,
// double or double-float) and runs every x and y line transform of the
// plane there: the band rows along x, all 120 columns along y, and for H psi
// the band rows back along x.  Between the z passes the plane never leaves
// the SM.  These kernels stand in for the x and y passes of
// FourierTransform::bwd / fwd (FourierTransform.cc:584-1362) on the
// 120 x 120 planes of the 216-atom cell's grid.
//
// Each 120-point line runs as an in-place, in-order prime-factor transform
// (Burrus and Eschenbacher, 1981): the same Ruritanian map
//     n = (15 n1 + 40 a + 24 b) mod 120,   n1 < 8, a < 3, b < 5
// indexes both the input and the output.  Then
//     n k = 105 n1 k1 + 40 a ka + 96 b kb  (mod 120),
// so, for the direction s (exp(s 2 pi i n k / 120)), the transform is a
// 3-point DFT over a with the root exp(s 2 pi i / 3), a 5-point DFT over b
// with exp(s 2 pi i 4/5) = exp(-s 2 pi i / 5) and an 8-point DFT over n1
// with exp(s 2 pi i 7/8) = exp(-s 2 pi i / 8): the opposite-direction 5- and
// 8-point codelets.  Every item of every pass reads and writes the same
// slots, so items are independent within a pass, the passes commute, and
// the 8-point items on either side of a pointwise product (the local
// potential of H psi) are one register-resident item.  The 8-point items of
// the last backward pass hand their outputs straight to memory (density,
// real-space fields), and in the adjoint's H applications pair the
// backward transform with a stored field before the v(r) product.
//
// Shared-memory banks: rows are 121 elements apart, so 8 consecutive rows
// at one x (row passes, rows fastest across threads) and 8 consecutive x at
// one y (column passes, columns fastest) fall on 8 distinct 16-byte bank
// groups.
#include <algorithm>

#include "qbg_internal.h"

namespace qbg {

constexpr int kPl = 120;         // plane side
constexpr int kPlLs = kPl + 1;   // row stride in shared memory (elements)
// threads per CTA: 768 = 24 warps at 80 registers per thread
#ifndef QBG_PL_THREADS
#define QBG_PL_THREADS 768
#endif
constexpr int kPlThreads = QBG_PL_THREADS;
constexpr size_t kPlane = (size_t)kPl * kPl;
template <typename T> constexpr size_t plane_smem_bytes() {
  return sizeof(cplx<T>) * (size_t)kPl * kPlLs;
}
// density and pair-product slots: FP64 for FP64 transforms, double-float
// for double-float ones
template <typename T> struct PlSlot { using type = double; };
template <> struct PlSlot<df32> { using type = df32; };

template <typename T> __device__ __forceinline__ cplx<T> pl_zero() {
  cplx<T> c;
  c.x = T(0);
  c.y = T(0);
  return c;
}
// floor(a / b) for 0 <= a < 2^20, 1 <= b <= 4096, inv = 1/b in FP32
__device__ __forceinline__ int pl_div(int a, float inv) { return (int)(((float)a + 0.5f) * inv); }

template <typename T> __device__ __forceinline__ double pl_to_f64(T x) { return (double)x; }
template <> __device__ __forceinline__ double pl_to_f64<df32>(df32 x) { return f64_from_df32(x); }
template <typename T> __device__ __forceinline__ T pl_from_f64(double x) { return (T)x; }
template <> __device__ __forceinline__ df32 pl_from_f64<df32>(double x) { return df32_from_f64(x); }

// pass P over the plane's band rows (b < ntr: y = b, else y = b + 120 -
// nband), rows fastest across threads; ends with a barrier
template <int P, int S, typename C>
__device__ __forceinline__ void pl_rows(C* Pl, int nband, int ntr, float inb) {
  constexpr int NI = PlPass<P>::NI;
  for (int it = threadIdx.x; it < nband * NI; it += blockDim.x) {
    const int j = pl_div(it, inb), b = it - j * nband;
    const int y = b < ntr ? b : b + (kPl - nband);
    pl_item<P, S, 1>(Pl + y * kPlLs, j);
  }
  __syncthreads();
}

// pass P over all 120 columns, columns fastest across threads; ends with a
// barrier
template <int P, int S, typename C> __device__ __forceinline__ void pl_cols(C* Pl) {
  constexpr int NI = PlPass<P>::NI;
  for (int it = threadIdx.x; it < kPl * NI; it += blockDim.x) {
    const int j = it / kPl, x = it - j * kPl;
    pl_item<P, S, kPlLs>(Pl + x, j);
  }
  __syncthreads();
}

// all three passes of the band rows' x transform (direction S)
template <int S, typename C>
__device__ __forceinline__ void pl_rows_all(C* Pl, int nband, int ntr, float inb) {
  if constexpr (S > 0) {
    pl_rows<0, S>(Pl, nband, ntr, inb);
    pl_rows<1, S>(Pl, nband, ntr, inb);
    pl_rows<2, S>(Pl, nband, ntr, inb);
  } else {
    pl_rows<2, S>(Pl, nband, ntr, inb);
    pl_rows<1, S>(Pl, nband, ntr, inb);
    pl_rows<0, S>(Pl, nband, ntr, inb);
  }
}

// plane <- rods of Zr in band-row order (zeros elsewhere); ends with a barrier
template <typename T>
__device__ __forceinline__ void pl_fill(cplx<T>* Pl, const cplx<T>* __restrict__ Zr, int nrods,
                                        const int* __restrict__ row_rod,
                                        const int* __restrict__ row_xb, int nband, int ntr) {
  using C = cplx<T>;
  const C zero = pl_zero<T>();
  for (int i = threadIdx.x; i < kPl * kPlLs; i += blockDim.x) Pl[i] = zero;
  __syncthreads();
  // four rods per thread per round: all loads issued before the stores
  for (int q0 = threadIdx.x; q0 < nrods; q0 += 4 * blockDim.x) {
    int xb[4];
    C val[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int q = q0 + u * blockDim.x;
      xb[u] = q < nrods ? row_xb[q] : -1;
      if (q < nrods) val[u] = Zr[row_rod[q]];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (xb[u] < 0) continue;
      const int b = xb[u] >> 16, y = b < ntr ? b : b + (kPl - nband);
      Pl[y * kPlLs + (xb[u] & 0xffff)] = val[u];
    }
  }
  __syncthreads();
}

// Z row of rods -> x backward -> y passes 3 and 5 backward; the caller runs
// the 8-point items of the last y pass
template <typename T>
__device__ __forceinline__ void pl_backward_to_last(cplx<T>* Pl, const cplx<T>* Zr, int nrods,
                                                    const int* row_rod, const int* row_xb,
                                                    int nband) {
  const int ntr = nband / 2 + (nband & 1);
  const float inb = 1.f / (float)nband;
  pl_fill<T>(Pl, Zr, nrods, row_rod, row_xb, nband, ntr);
  pl_rows_all<+1>(Pl, nband, ntr, inb);
  pl_cols<0, +1>(Pl);
  pl_cols<1, +1>(Pl);
}

// 16-byte asynchronous copies global -> shared (cp.async: the hardware
// completes them, no wait loop of ours)
__device__ __forceinline__ void pl_cp16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(
                   (unsigned)__cvta_generic_to_shared(dst)),
               "l"(src));
}
__device__ __forceinline__ void pl_cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void pl_cp_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// H psi middle for (plane z, state s) work items w = z + n2 s: Z row of rods
// -> x backward -> y backward -> v(r) product -> y forward -> x forward -> Z
// row of rods.  v holds the plane-major local potential in the transform
// arithmetic T.  Persistent CTAs walk the items with a grid stride.  With
// STAGE (the Z row fits in the plane's non-band rows), the next
// item's Z row is copied into the non-band rows while the x forward passes
// of the current one run there on the band rows only, so the next plane
// fills from shared memory instead of waiting on HBM.
//
// With PAIR, the backward transform psi(r) that the 8-point items hold just
// before the v(r) product is also paired with a stored real-space field:
// slot[w][r] = Re(conj(psi(r)) G(r)) (the adjoint's dL/dv term of this
// H application; G and the slots are [state][z][y][x] of this chunk).
template <typename T, bool STAGE, bool PAIR>
__global__ void __launch_bounds__(kPlThreads, 1)
k_plane_vloc(cplx<T>* __restrict__ Z, int nrods, const int* __restrict__ row_rod,
             const int* __restrict__ row_xb, int nband, int n2, int ns,
             const T* __restrict__ v, const cplx<T>* __restrict__ G,
             typename PlSlot<T>::type* __restrict__ slots) {
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem[];
  C* Pl = reinterpret_cast<C*>(smem);
  const int ntr = nband / 2 + (nband & 1);
  const int nlow = ntr, nhigh = kPl - (nband - ntr);  // non-band rows [nlow, nhigh)
  const float inb = 1.f / (float)nband;
  C* Sg = Pl + nlow * kPlLs;  // staging: the Z row in rod order
  const int W = n2 * ns;
  int w = blockIdx.x;
  if (STAGE && w < W) {
    const C* Zr = Z + (size_t)w * nrods;
    for (int q = threadIdx.x; q < nrods; q += blockDim.x) pl_cp16(Sg + q, Zr + q);
    pl_cp_commit();
  }
  for (; w < W; w += gridDim.x) {
    const int z = w % n2;
    C* Zr = Z + (size_t)w * nrods;  // Z[s][z][rod] with w = z + n2 s
    const T* vz = v + (size_t)z * kPlane;
    if constexpr (STAGE) {
      const C zero = pl_zero<T>();
      for (int i = threadIdx.x; i < nband * kPlLs; i += blockDim.x) {
        const int b = i / kPlLs;
        Pl[(b < ntr ? i : i + (nhigh - nlow) * kPlLs)] = zero;
      }
      pl_cp_wait_all();
      __syncthreads();
      for (int q = threadIdx.x; q < nrods; q += blockDim.x) {
        const int xb = row_xb[q];
        const int b = xb >> 16, y = b < ntr ? b : b + (kPl - nband);
        Pl[y * kPlLs + (xb & 0xffff)] = Sg[row_rod[q]];
      }
      __syncthreads();
      // the non-band rows are zeroed alongside the first x pass, which does
      // not touch them
      for (int i = threadIdx.x; i < (nhigh - nlow) * kPlLs; i += blockDim.x) Sg[i] = zero;
      pl_rows<0, +1>(Pl, nband, ntr, inb);
      pl_rows<1, +1>(Pl, nband, ntr, inb);
      pl_rows<2, +1>(Pl, nband, ntr, inb);
      pl_cols<0, +1>(Pl);
      pl_cols<1, +1>(Pl);
    } else {
      pl_backward_to_last<T>(Pl, Zr, nrods, row_rod, row_xb, nband);
    }
    // 8-point items: backward, v(r) product, forward, in registers
    for (int it = threadIdx.x; it < kPl * 15; it += blockDim.x) {
      const int j = it / kPl, x = it - j * kPl;
      int i[8];
      pl_slots<2>(j, i);
      T vv[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) vv[k] = vz[i[k] * kPl + x];
      C u[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) u[k] = Pl[i[k] * kPlLs + x];
      pl_dft<2, +1>(u);
      if constexpr (PAIR) {
        const cplx<T>* Gz = G + (size_t)w * kPlane;
        typename PlSlot<T>::type* rz = slots + (size_t)w * kPlane;
        // two halves of four keep the field loads within 80 registers
#pragma unroll
        for (int h = 0; h < 8; h += 4) {
          cplx<T> g[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) g[k] = Gz[i[h + k] * kPl + x];
#pragma unroll
          for (int k = 0; k < 4; ++k)
            rz[i[h + k] * kPl + x] = u[h + k].x * g[k].x + u[h + k].y * g[k].y;
        }
      }
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        u[k].x = u[k].x * vv[k];
        u[k].y = u[k].y * vv[k];
      }
      pl_dft<2, -1>(u);
#pragma unroll
      for (int k = 0; k < 8; ++k) Pl[i[k] * kPlLs + x] = u[k];
    }
    __syncthreads();
    pl_cols<1, -1>(Pl);
    pl_cols<0, -1>(Pl);
    // the non-band rows are free from here on: stage the next item's Z row
    const int wn = w + gridDim.x;
    if (STAGE && wn < W) {
      const C* Zn = Z + (size_t)wn * nrods;
      for (int q = threadIdx.x; q < nrods; q += blockDim.x) pl_cp16(Sg + q, Zn + q);
      pl_cp_commit();
    }
    pl_rows_all<-1>(Pl, nband, ntr, inb);
    for (int q = threadIdx.x; q < nrods; q += blockDim.x) {
      const int xb = row_xb[q];
      const int b = xb >> 16, y = b < ntr ? b : b + (kPl - nband);
      Zr[row_rod[q]] = Pl[y * kPlLs + (xb & 0xffff)];
    }
    __syncthreads();  // the band rows are read above before the next fill
  }
  pl_cp_wait_all();
}

// Output of the last backward pass, per 8-point item of column x.
// Density: slot s (+)= w_s |psi(r)|^2.
template <typename T> struct PlDensity {
  using ST = typename PlSlot<T>::type;
  ST* rz;
  T ws;
  int accumulate;
  __device__ __forceinline__ void operator()(const cplx<T>* u, const int* i, int x) const {
    ST old[8];
    if (accumulate) {
#pragma unroll
      for (int k = 0; k < 8; ++k) old[k] = rz[i[k] * kPl + x];
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const T a = ws * (u[k].x * u[k].x + u[k].y * u[k].y);
      rz[i[k] * kPl + x] = accumulate ? old[k] + a : a;
    }
  }
};
// Real-space field: f = psi(r), FP64 (double2) or the transform type
template <typename T, typename OUT> struct PlField {
  OUT* fz;
  __device__ __forceinline__ void operator()(const cplx<T>* u, const int* i, int x) const {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      OUT o;
      if constexpr (std::is_same<OUT, double2>::value) {
        o.x = pl_to_f64(u[k].x);
        o.y = pl_to_f64(u[k].y);
      } else {
        o = u[k];
      }
      fz[i[k] * kPl + x] = o;
    }
  }
};
// Backward transform of one (plane z, state s) whose last pass hands each
// 8-point item's outputs to out (a PlDensity, PlField or PlPair bound to
// this plane and state).
template <typename T, typename OUT>
__device__ __forceinline__ void pl_backward(cplx<T>* Pl, const cplx<T>* Zr, int nrods,
                                            const int* row_rod, const int* row_xb, int nband,
                                            const OUT& out) {
  using C = cplx<T>;
  pl_backward_to_last<T>(Pl, Zr, nrods, row_rod, row_xb, nband);
  for (int it = threadIdx.x; it < kPl * 15; it += blockDim.x) {
    const int j = it / kPl, x = it - j * kPl;
    int i[8];
    pl_slots<2>(j, i);
    C u[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) u[k] = Pl[i[k] * kPlLs + x];
    pl_dft<2, +1>(u);
    out(u, i, x);
  }
}

template <typename T>
__global__ void __launch_bounds__(kPlThreads, 1)
k_plane_density(const cplx<T>* __restrict__ Z, int nrods, const int* __restrict__ row_rod,
                const int* __restrict__ row_xb, int nband, int n2,
                const double* __restrict__ w, typename PlSlot<T>::type* __restrict__ slots,
                int accumulate) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int z = blockIdx.x, s = blockIdx.y;
  PlDensity<T> out{slots + ((size_t)s * n2 + z) * kPlane, T(w[s]), accumulate};
  pl_backward<T>(reinterpret_cast<cplx<T>*>(smem), Z + ((size_t)s * n2 + z) * nrods, nrods,
                 row_rod, row_xb, nband, out);
}

template <typename T, typename OUT>
__global__ void __launch_bounds__(kPlThreads, 1)
k_plane_field(const cplx<T>* __restrict__ Z, int nrods, const int* __restrict__ row_rod,
              const int* __restrict__ row_xb, int nband, int n2, OUT* __restrict__ f) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int z = blockIdx.x, s = blockIdx.y;
  PlField<T, OUT> out{f + ((size_t)s * n2 + z) * kPlane};
  pl_backward<T>(reinterpret_cast<cplx<T>*>(smem), Z + ((size_t)s * n2 + z) * nrods, nrods,
                 row_rod, row_xb, nband, out);
}

// Forward transform of one (plane z, state s) from an FP64 real-space field
// f[s][z][y][x]: the first y pass (8-point items) reads f straight from
// memory, the x passes run on the band rows only, the rods go to Z.
template <typename T>
__global__ void __launch_bounds__(kPlThreads, 1)
k_plane_fwd(const double2* __restrict__ f, cplx<T>* __restrict__ Z, int nrods,
            const int* __restrict__ row_rod, const int* __restrict__ row_xb, int nband, int n2) {
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem[];
  C* Pl = reinterpret_cast<C*>(smem);
  const int z = blockIdx.x, s = blockIdx.y;
  const int ntr = nband / 2 + (nband & 1);
  const float inb = 1.f / (float)nband;
  const double2* fz = f + ((size_t)s * n2 + z) * kPlane;
  for (int it = threadIdx.x; it < kPl * 15; it += blockDim.x) {
    const int j = it / kPl, x = it - j * kPl;
    int i[8];
    pl_slots<2>(j, i);
    double2 g[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) g[k] = fz[i[k] * kPl + x];
    C u[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      u[k].x = pl_from_f64<T>(g[k].x);
      u[k].y = pl_from_f64<T>(g[k].y);
    }
    pl_dft<2, -1>(u);
#pragma unroll
    for (int k = 0; k < 8; ++k) Pl[i[k] * kPlLs + x] = u[k];
  }
  __syncthreads();
  pl_cols<1, -1>(Pl);
  pl_cols<0, -1>(Pl);
  pl_rows_all<-1>(Pl, nband, ntr, inb);
  C* Zr = Z + ((size_t)s * n2 + z) * nrods;
  for (int q = threadIdx.x; q < nrods; q += blockDim.x) {
    const int xb = row_xb[q];
    const int b = xb >> 16, y = b < ntr ? b : b + (kPl - nband);
    Zr[row_rod[q]] = Pl[y * kPlLs + (xb & 0xffff)];
  }
}

// grad[r] += scale * sum_{s < ns} slot[s][r], slots in state order
// (deterministic)
template <typename ST>
__global__ void __launch_bounds__(256)
k_plane_slot_sum(const ST* __restrict__ slots, int ns, long long n, double scale,
                 double* __restrict__ grad) {
  // the sum runs in the slots' type (double-float on the FP32 pipe), the
  // loads of eight slots issued before their adds
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (long long)gridDim.x * blockDim.x) {
    ST a = slots[r];
    for (int s0 = 1; s0 < ns; s0 += 8) {
      ST v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (s0 + u < ns) v[u] = slots[(size_t)(s0 + u) * n + r];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (s0 + u < ns) a = a + v[u];
    }
    grad[r] += scale * pl_to_f64(a);
  }
}

// ------------------------------------------------------------- launchers
template <typename K> static cudaError_t pl_prep(K kernel, size_t smem) {
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

bool plane_applies(const qbg_plan* p, bool fp32) {
  return !fp32 && p->fuse_xyx && p->plane_xyx && p->np0 == kPl && p->np1 == kPl &&
         p->len[0].allow_pfa && p->len[1].allow_pfa;
}

template <typename T> qbg_status plane_vloc(qbg_plan* p, int ns, int s0, cudaStream_t st) {
  using ST = typename PlSlot<T>::type;
  const size_t sm = plane_smem_bytes<T>();
  QBG_CUDA(pl_prep(k_plane_vloc<T, true, false>, sm));
  QBG_CUDA(pl_prep(k_plane_vloc<T, false, false>, sm));
  QBG_CUDA(pl_prep(k_plane_vloc<T, true, true>, sm));
  QBG_CUDA(pl_prep(k_plane_vloc<T, false, true>, sm));
  const T* v = std::is_same<T, double>::value ? (const T*)p->d_vr : (const T*)p->d_vrdf;
  // one persistent CTA per SM; the Z row is staged in the non-band rows when
  // it fits there
  if (!p->nsm) {
    int dev = 0;
    QBG_CUDA(cudaGetDevice(&dev));
    QBG_CUDA(cudaDeviceGetAttribute(&p->nsm, cudaDevAttrMultiProcessorCount, dev));
  }
  const int nsm = p->nsm;
  const int W = p->np2 * ns;
  const bool stage = (size_t)p->nrods <= (size_t)(kPl - p->nband) * kPlLs;
  const int grid = std::min(W, std::max(nsm, 1));
  // the adjoint's pairing context (set around an H application)
  const bool pair = p->pair_G != nullptr;
  const cplx<T>* G = pair ? (const cplx<T>*)p->pair_G + (size_t)s0 * p->N : nullptr;
  ST* slots = (ST*)p->pair_slots;
  {
    PhaseTimer pt(p, PH_XYX_VLOC, st);
    auto* k = stage ? (pair ? k_plane_vloc<T, true, true> : k_plane_vloc<T, true, false>)
                    : (pair ? k_plane_vloc<T, false, true> : k_plane_vloc<T, false, false>);
    k<<<grid, kPlThreads, sm, st>>>((cplx<T>*)p->d_Z, p->nrods, p->d_row_rod, p->d_row_x,
                                    p->nband, p->np2, ns, v, G, slots);
    QBG_LAUNCHED(p);
  }
  if (pair) {
    PhaseTimer pt(p, PH_XY_PAIR, st);
    k_plane_slot_sum<ST><<<2 * 152 * 4, 256, 0, st>>>(slots, ns, p->N, p->pair_scale,
                                                      p->pair_grad);
    QBG_LAUNCHED(p);
  }
  return QBG_OK;
}

template <typename T>
qbg_status plane_density(qbg_plan* p, int ns, const double* w, int acc, void* slots,
                         cudaStream_t st) {
  const size_t sm = plane_smem_bytes<T>();
  QBG_CUDA(pl_prep(k_plane_density<T>, sm));
  PhaseTimer pt(p, PH_Y_DENSITY, st);
  k_plane_density<T><<<dim3(p->np2, ns), kPlThreads, sm, st>>>(
      (const cplx<T>*)p->d_Z, p->nrods, p->d_row_rod, p->d_row_x, p->nband, p->np2, w,
      (typename PlSlot<T>::type*)slots, acc);
  QBG_LAUNCHED(p);
  return QBG_OK;
}

template <typename T>
qbg_status plane_field(qbg_plan* p, int ns, double2* f, cudaStream_t st) {
  const size_t sm = plane_smem_bytes<T>();
  QBG_CUDA(pl_prep(k_plane_field<T, double2>, sm));
  PhaseTimer pt(p, PH_Y_STORE, st);
  k_plane_field<T, double2><<<dim3(p->np2, ns), kPlThreads, sm, st>>>(
      (const cplx<T>*)p->d_Z, p->nrods, p->d_row_rod, p->d_row_x, p->nband, p->np2, f);
  QBG_LAUNCHED(p);
  return QBG_OK;
}

template <typename T>
qbg_status plane_fwd(qbg_plan* p, int ns, const double2* f, cudaStream_t st) {
  const size_t sm = plane_smem_bytes<T>();
  QBG_CUDA(pl_prep(k_plane_fwd<T>, sm));
  PhaseTimer pt(p, PH_Y_LOAD, st);
  k_plane_fwd<T><<<dim3(p->np2, ns), kPlThreads, sm, st>>>(
      f, (cplx<T>*)p->d_Z, p->nrods, p->d_row_rod, p->d_row_x, p->nband, p->np2);
  QBG_LAUNCHED(p);
  return QBG_OK;
}

template <typename T>
qbg_status plane_pair_field(qbg_plan* p, int ns, void* F, cudaStream_t st) {
  const size_t sm = plane_smem_bytes<T>();
  QBG_CUDA(pl_prep(k_plane_field<T, cplx<T>>, sm));
  PhaseTimer pt(p, PH_XY_PAIR, st);
  k_plane_field<T, cplx<T>><<<dim3(p->np2, ns), kPlThreads, sm, st>>>(
      (const cplx<T>*)p->d_Z, p->nrods, p->d_row_rod, p->d_row_x, p->nband, p->np2,
      (cplx<T>*)F);
  QBG_LAUNCHED(p);
  return QBG_OK;
}

#define QBG_PLANE_INST(T)                                                                      \
  template qbg_status plane_vloc<T>(qbg_plan*, int, int, cudaStream_t);                        \
  template qbg_status plane_density<T>(qbg_plan*, int, const double*, int, void*,              \
                                       cudaStream_t);                                          \
  template qbg_status plane_field<T>(qbg_plan*, int, double2*, cudaStream_t);                  \
  template qbg_status plane_fwd<T>(qbg_plan*, int, const double2*, cudaStream_t);              \
  template qbg_status plane_pair_field<T>(qbg_plan*, int, void*, cudaStream_t);
QBG_PLANE_INST(double)
QBG_PLANE_INST(df32)

}  // namespace qbg
