// qbg_graph.cu -- many independent cells stepped as one CUDA graph, and the
// chunk-size autotuner.
//
// A batch is a list of plans (cells of any grid, basis and state count),
// each with its own psi.  qbg_etrs_graph_create captures one ETRS step of
// every cell into a single CUDA graph: the cells are forked onto their own
// streams inside the capture, so the graph holds one independent branch per
// cell and the GPU runs them concurrently; replaying the graph steps all
// cells with one launch call and no per-kernel launch overhead.  Before the
// capture one uncaptured step runs on scratch copies of the states, so every
// work buffer exists and every table is built (a capture may not allocate,
// synchronise or copy to the host); the per-step tensor-core status read is
// left out of the capture and done by qbg_etrs_graph_check.
#include <algorithm>
#include <vector>

#include "qbg_internal.h"

struct qbg_graph {
  std::vector<qbg_plan*> plans;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace qbg {

#define QBG_TRY(x)                \
  do {                            \
    qbg_status s_ = (x);          \
    if (s_ != QBG_OK) return s_;  \
  } while (0)

static void graph_free(qbg_graph* g) {
  if (!g) return;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  for (cudaStream_t s : g->streams)
    if (s) cudaStreamDestroy(s);
  for (cudaEvent_t e : g->joins)
    if (e) cudaEventDestroy(e);
  if (g->fork) cudaEventDestroy(g->fork);
  delete g;
}

}  // namespace qbg

using namespace qbg;

extern "C" {

qbg_status qbg_etrs_graph_create(int ncells, qbg_plan* const* plans, double* const* psi,
                                 const int* ld, const int* nst, const double* const* occ,
                                 double dt, void* stream, qbg_graph** out) {
  if (!out || ncells <= 0 || !plans || !psi || !ld || !nst || !occ) {
    set_error("qbg_etrs_graph_create: invalid argument");
    return QBG_ERR_INVALID;
  }
  *out = nullptr;
  for (int i = 0; i < ncells; ++i) {
    if (!plans[i] || !psi[i] || nst[i] <= 0 || ld[i] < plans[i]->ngw || !occ[i]) {
      set_error("qbg_etrs_graph_create: cell %d: invalid argument", i);
      return QBG_ERR_INVALID;
    }
    for (int j = 0; j < i; ++j)
      if (plans[j] == plans[i]) {
        set_error("qbg_etrs_graph_create: cell %d repeats the plan of cell %d", i, j);
        return QBG_ERR_INVALID;
      }
  }
  // a capture cannot run on the legacy default stream: use an internal one
  cudaStream_t origin = (cudaStream_t)stream;
  cudaStream_t own = nullptr;
  if (!origin) {
    QBG_CUDA(cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking));
    origin = own;
  }
  struct OwnGuard {
    cudaStream_t s;
    ~OwnGuard() {
      if (s) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
      }
    }
  } guard{own};
  qbg_graph* g = new qbg_graph;
  g->plans.assign(plans, plans + ncells);
  auto fail = [&](qbg_status s) {
    graph_free(g);
    return s;
  };
  // warm-up step on scratch copies: every buffer and table of the step exists
  // afterwards, and the per-state factors are cached for the same occupations
  for (int i = 0; i < ncells; ++i) {
    qbg_plan* p = plans[i];
    const size_t bytes = sizeof(double2) * (size_t)ld[i] * nst[i];
    double* tmp = nullptr;
    cudaError_t e = cudaMalloc(&tmp, bytes);
    if (e == cudaSuccess) e = cudaMemcpyAsync(tmp, psi[i], bytes, cudaMemcpyDeviceToDevice, origin);
    if (e != cudaSuccess) {
      if (tmp) cudaFree(tmp);
      return fail(cuda_status(e, "qbg_etrs_graph_create"));
    }
    qbg_status s = qbg_etrs_step(p, tmp, ld[i], nst[i], occ[i], dt, nullptr, nullptr, nullptr,
                                 nullptr, origin);
    cudaStreamSynchronize(origin);
    cudaFree(tmp);
    if (s != QBG_OK) return fail(s);
  }
  // capture: fork one stream per cell off the origin stream, join back
  cudaError_t e = cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming);
  if (e != cudaSuccess) return fail(cuda_status(e, "qbg_etrs_graph_create"));
  g->streams.assign(ncells, nullptr);
  g->joins.assign(ncells, nullptr);
  for (int i = 0; i < ncells; ++i) {
    e = cudaStreamCreateWithFlags(&g->streams[i], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->joins[i], cudaEventDisableTiming);
    if (e != cudaSuccess) return fail(cuda_status(e, "qbg_etrs_graph_create"));
  }
  std::vector<bool> check(ncells);
  for (int i = 0; i < ncells; ++i) {
    check[i] = plans[i]->check_every_step;
    plans[i]->check_every_step = false;  // the status is read by qbg_etrs_graph_check
  }
  qbg_status st = QBG_OK;
  e = cudaStreamBeginCapture(origin, cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) {
    cudaEventRecord(g->fork, origin);
    for (int i = 0; i < ncells && st == QBG_OK; ++i) {
      cudaStreamWaitEvent(g->streams[i], g->fork, 0);
      st = qbg_etrs_step(plans[i], psi[i], ld[i], nst[i], occ[i], dt, nullptr, nullptr, nullptr,
                         nullptr, g->streams[i]);
      cudaEventRecord(g->joins[i], g->streams[i]);
      cudaStreamWaitEvent(origin, g->joins[i], 0);
    }
    const cudaError_t e2 = cudaStreamEndCapture(origin, &g->graph);
    if (e2 != cudaSuccess && st == QBG_OK) st = cuda_status(e2, "cudaStreamEndCapture");
  } else {
    st = cuda_status(e, "cudaStreamBeginCapture");
  }
  for (int i = 0; i < ncells; ++i) plans[i]->check_every_step = check[i];
  if (st != QBG_OK) return fail(st);
  e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  if (e != cudaSuccess) return fail(cuda_status(e, "cudaGraphInstantiate"));
  *out = g;
  return QBG_OK;
}

qbg_status qbg_etrs_graph_launch(qbg_graph* g, void* stream) {
  if (!g || !g->exec) {
    set_error("qbg_etrs_graph_launch: null graph");
    return QBG_ERR_INVALID;
  }
  QBG_CUDA(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
  return QBG_OK;
}

qbg_status qbg_etrs_graph_check(qbg_graph* g) {
  if (!g) {
    set_error("qbg_etrs_graph_check: null graph");
    return QBG_ERR_INVALID;
  }
  QBG_CUDA(cudaDeviceSynchronize());
  for (qbg_plan* p : g->plans) QBG_TRY(tc_check_status(p, nullptr));
  return QBG_OK;
}

qbg_status qbg_etrs_graph_destroy(qbg_graph* g) {
  graph_free(g);
  return QBG_OK;
}

qbg_status qbg_plan_autotune(qbg_plan* p, const double* psi, int ld, int nst, const double* occ,
                             void* stream, int* chosen) {
  if (!p || !psi || nst <= 0 || ld < p->ngw) {
    set_error("qbg_plan_autotune: invalid argument");
    return QBG_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  double* out = nullptr;
  QBG_CUDA(cudaMalloc(&out, sizeof(double2) * (size_t)ld * nst));
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  qbg_status s = QBG_OK;
  // device time of two H|psi> after a warm-up (which also grows the scratch)
  auto time_h = [&](float* ms) -> qbg_status {
    qbg_status r = qbg_hpsi(p, psi, ld, out, nst, occ, nullptr, stream);
    if (r != QBG_OK) return r;
    cudaEventRecord(a, st);
    for (int k = 0; k < 2 && r == QBG_OK; ++k) r = qbg_hpsi(p, psi, ld, out, nst, occ, nullptr, stream);
    cudaEventRecord(b, st);
    cudaEventSynchronize(b);
    *ms = 0.f;
    cudaEventElapsedTime(ms, a, b);
    return r;
  };
  int cfg0[5];
  qbg_plan_get_transform_config(p, cfg0);
  // 1) transform shape at the current chunk: radix order of the Stockham
  //    passes, prime-factor splits, the fused x-y-x kernel, the
  //    register lane-group y pass (FP32 transforms only)
  int best[4] = {cfg0[1], cfg0[2], cfg0[3], cfg0[4]};
  float best_ms = 1e30f;
  const bool fp32 = p->prec == QBG_PREC_MIXED || p->prec == QBG_PREC_MIXED_NL64;
  for (int order = 0; order < 3 && s == QBG_OK; ++order)
    for (int pfa = 1; pfa >= 0 && s == QBG_OK; --pfa)
      for (int fused = 2; fused >= 0 && s == QBG_OK; --fused)
        for (int lane = 1; lane >= (fp32 ? 0 : 1) && s == QBG_OK; --lane) {
          if (!pfa && fused) continue;  // the fused kernels need the prime-factor splits
          // the whole-plane kernel: 120 x 120 planes, FP64 or double-float
          if (fused == 2 && (fp32 || p->np0 != 120 || p->np1 != 120)) continue;
          s = qbg_plan_set_transform_config(p, order, pfa, fused, lane);
          float ms = 0.f;
          if (s == QBG_OK) s = time_h(&ms);
          if (s == QBG_OK && ms < best_ms) {
            best_ms = ms;
            best[0] = order;
            best[1] = pfa;
            best[2] = fused;
            best[3] = lane;
          }
        }
  if (s == QBG_OK) s = qbg_plan_set_transform_config(p, best[0], best[1], best[2], best[3]);
  // 2) states per transform launch group with that shape
  int best_ch = cfg0[0];
  best_ms = 1e30f;
  for (int ch : {8, 16, 32, 64, 96, 144}) {
    if (s != QBG_OK || (ch > 2 * nst && ch != 8)) break;
    p->chunk = ch;
    float ms = 0.f;
    s = time_h(&ms);
    if (s == QBG_OK && ms < best_ms) {
      best_ms = ms;
      best_ch = ch;
    }
  }
  if (s == QBG_OK) {
    p->chunk = best_ch;
  } else {
    p->chunk = cfg0[0];
    qbg_plan_set_transform_config(p, cfg0[1], cfg0[2], cfg0[3], cfg0[4]);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  if (chosen) *chosen = p->chunk;
  return s;
}

}  // extern "C"
