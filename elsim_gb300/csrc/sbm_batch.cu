// sbm_batch.cu -- many independent sub-volume solves in one graph launch.
//
// Every sub-volume keeps its own context (fields, FP32 work, CG state and
// captured iteration chunk).  The batch driver starts each volume's
// mixed-precision solve (set-up kernels on the volume's stream), then builds
// one parent CUDA graph whose child nodes are the volumes' iteration-chunk
// graphs: a single cudaGraphLaunch advances every volume by one chunk, the
// volumes' kernels running side by side on the GPU, and volumes that have
// converged turn into no-ops through their own `done` flag.  The host reads
// all volume states after each round (one pinned copy each) while the next
// round is already queued.  No counterpart in the reference, which solves one
// domain per MPI job.
#include <cstring>
#include <string>
#include <vector>

#include "sbm_internal.cuh"

using namespace sbm;

namespace sbm {
int ghost_after_solve(sbm_ctx* ctx, double* f, int bcx0, int bcx1);  // sbm_fields.cu
}

namespace {

struct BatchCache {
  std::string key;
  cudaGraph_t parent = nullptr;
  cudaGraphExec_t exec = nullptr;
  int nodes = 0;
};
BatchCache g_batch;

}  // namespace

extern "C" int sbm_batch_solve(sbm_ctx** ctxs, int n, int bc_x0, int bc_x1, double scale,
                               double tol, int max_it, int precond, int* iters, double* final_res,
                               int* status, float* ms_total) {
  if (!ctxs || n < 1 || max_it < 1 || !(tol >= 0.0)) return SBM_ERR_ARG;
  if ((bc_x0 != SBM_BC_COPY && bc_x0 != SBM_BC_ZERO) || (bc_x1 != SBM_BC_COPY && bc_x1 != SBM_BC_ZERO) ||
      (precond != SBM_PC_NONE && precond != SBM_PC_JACOBI && precond != SBM_PC_LEARNED))
    return SBM_ERR_ARG;
  for (int v = 0; v < n; ++v)
    if (!ctxs[v]) return SBM_ERR_ARG;
  std::vector<SolveSpec> specs(n);
  std::vector<cudaGraph_t> graphs(n);
  cudaStream_t bs = ctxs[0]->stream;  // the batch runs on the first volume's stream
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  SBM_CUDA_TRY(cudaEventCreate(&t0));
  SBM_CUDA_TRY(cudaEventCreate(&t1));
  SBM_CUDA_TRY(cudaEventRecord(t0, bs));
  std::string key;
  int nodes_total = 0;
  for (int v = 0; v < n; ++v) {
    sbm_ctx* c = ctxs[v];
    SBM_CUDA_TRY(cudaStreamWaitEvent(c->stream, t0, 0));
    int rc = generic_spec(c, bc_x0, bc_x1, scale, tol, max_it, SBM_STOP_REL_RES, SBM_PREC_MIXED,
                          precond, &specs[v]);
    if (rc) return rc;
    cudaGraphExec_t ex = nullptr;
    int nodes = 0;
    rc = mixed_begin(c, specs[v], &ex, &graphs[v], &nodes);
    if (rc) return rc;
    nodes_total += nodes;
    char buf[48];
    snprintf(buf, sizeof(buf), "%p,", (void*)graphs[v]);
    key += buf;
    // the batch stream waits for this volume's set-up
    cudaEvent_t e = c->evq[0];
    SBM_CUDA_TRY(cudaEventRecord(e, c->stream));
    SBM_CUDA_TRY(cudaStreamWaitEvent(bs, e, 0));
  }
  if (key != g_batch.key) {
    if (g_batch.exec) cudaGraphExecDestroy(g_batch.exec);
    if (g_batch.parent) cudaGraphDestroy(g_batch.parent);
    g_batch = BatchCache();
    SBM_CUDA_TRY(cudaGraphCreate(&g_batch.parent, 0));
    for (int v = 0; v < n; ++v) {
      cudaGraphNode_t node;
      SBM_CUDA_TRY(cudaGraphAddChildGraphNode(&node, g_batch.parent, nullptr, 0, graphs[v]));
    }
    SBM_CUDA_TRY(cudaGraphInstantiate(&g_batch.exec, g_batch.parent, 0));
    g_batch.key = key;
    g_batch.nodes = nodes_total;
  }
  // rounds: one parent launch per round, all states read back while the
  // next round is queued
  CgState* h = nullptr;
  SBM_CUDA_TRY(cudaMallocHost(&h, sizeof(CgState) * 2 * n));
  cudaEvent_t ev[2];
  SBM_CUDA_TRY(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
  SBM_CUDA_TRY(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
  int rc = SBM_OK;
  auto round = [&](int slot) -> int {
    SBM_CUDA_TRY(cudaGraphLaunch(g_batch.exec, bs));
    for (int v = 0; v < n; ++v)
      SBM_CUDA_TRY(cudaMemcpyAsync(&h[slot * n + v], ctxs[v]->st, sizeof(CgState),
                                   cudaMemcpyDeviceToHost, bs));
    SBM_CUDA_TRY(cudaEventRecord(ev[slot], bs));
    SBM_LAUNCHED(g_batch.nodes);
    return SBM_OK;
  };
  int last = 0;
  if ((rc = round(0)) == SBM_OK) {
    for (int r = 1;; ++r) {
      if ((rc = round(r & 1))) break;
      if (cudaEventSynchronize(ev[(r - 1) & 1]) != cudaSuccess) {
        rc = SBM_ERR_CUDA;
        break;
      }
      bool all = true;
      for (int v = 0; v < n && all; ++v) all = h[((r - 1) & 1) * n + v].done != 0;
      last = r & 1;
      if (all) break;
    }
  }
  if (rc == SBM_OK && cudaEventSynchronize(ev[last]) != cudaSuccess) rc = SBM_ERR_CUDA;
  if (rc == SBM_OK) {
    for (int v = 0; v < n && rc == SBM_OK; ++v) {
      sbm_ctx* c = ctxs[v];
      SBM_CUDA_TRY(cudaStreamWaitEvent(c->stream, ev[last], 0));
      SolveResult res{};
      rc = mixed_end(c, specs[v], h[last * n + v], &res);
      if (rc) break;
      // same post-condition as a single solve: Dirichlet faces keep their
      // data, the other ghosts copy the edge
      if ((rc = ghost_after_solve(c, specs[v].x, bc_x0, bc_x1))) break;
      if (iters) iters[v] = res.iters;
      if (final_res) final_res[v] = res.final_res;
      if (status) status[v] = res.status;
      cudaEvent_t e = c->evq[1];
      SBM_CUDA_TRY(cudaEventRecord(e, c->stream));
      SBM_CUDA_TRY(cudaStreamWaitEvent(bs, e, 0));
    }
  }
  SBM_CUDA_TRY(cudaEventRecord(t1, bs));
  SBM_CUDA_TRY(cudaEventSynchronize(t1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, t0, t1);
  if (ms_total) *ms_total = ms;
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFreeHost(h);
  return rc;
}
