// qbg_noalloc.cu -- the batched backward transform for callers that cannot
// allocate device memory at call time.
//
// Some callers of this library cannot call cudaMalloc when they run a
// transform: code that is being captured into a CUDA graph (device
// allocation is not an operation a stream capture can record), or a host
// application whose device memory is entirely owned by its own pool
// allocator, so that an allocation behind its back would fail or fragment
// the pool.  qbg_backward grows a plan-owned scratch buffer on demand;
// qbg_backward_noalloc instead takes its per-call scratch (the z-pass and
// x-pass intermediates) from one file-scope device array of fixed size that
// every GPU loading the library holds until the process exits.
#include <mutex>

#include "qbg_internal.h"

namespace qbg {

// 32 MiB: room for the intermediates of one state of a 120^3 transform with
// the 216-atom basis, or of several states of smaller grids.
constexpr size_t kNoAllocScratchBytes = 32ull << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 256;
static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[kMaxDevices];  // device address of the array, per device

// Device address of the static array on the current device.  The first call
// on a device resolves it with cudaGetSymbolAddress (host code cannot use the
// array's name as a device pointer) and keeps it for the life of the process,
// so the device must not be reset (cudaDeviceReset) between calls.
static qbg_status noalloc_scratch(void** out) {
  int dev = 0;
  QBG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("qbg_backward_noalloc: device ordinal %d out of range", dev);
    return QBG_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return cuda_status(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return QBG_OK;
}

}  // namespace qbg

using namespace qbg;

extern "C" qbg_status qbg_backward_noalloc(qbg_plan* p, const double* c, int ldc, double* f,
                                           int nbatch, void* stream) {
  if (!p || nbatch < 0 || ldc < p->ngw || (nbatch > 0 && (!c || !f))) {
    set_error("qbg_backward_noalloc: invalid argument");
    return QBG_ERR_INVALID;
  }
  if (nbatch == 0) return QBG_OK;
  // FP64 intermediates of one state: z pass [np2 x nrods], x pass
  // [np2 x nband x np0], each rounded up to 256 bytes
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t zb = up((size_t)p->np2 * p->nrods * sizeof(double2));
  const size_t yb = up((size_t)p->np2 * p->nband * p->np0 * sizeof(double2));
  if (zb + yb > kNoAllocScratchBytes) {
    set_error("qbg_backward_noalloc: one state needs %zu bytes of scratch; the static scratch "
              "holds %zu bytes (use qbg_backward)",
              zb + yb, (size_t)kNoAllocScratchBytes);
    return QBG_ERR_INVALID;
  }
  void* base = nullptr;
  qbg_status s = noalloc_scratch(&base);
  if (s != QBG_OK) return s;
  const int chunk = (int)std::min<size_t>((size_t)nbatch, kNoAllocScratchBytes / (zb + yb));
  unsigned char* Z = (unsigned char*)base;
  unsigned char* Y = Z + up(chunk * zb);
  return backward_scratch<double>(p, (const double2*)c, ldc, (double2*)f, nbatch, Z, Y, chunk,
                                  (cudaStream_t)stream);
}
