// sbm_batch.cu -- many independent sub-volume solves in one graph launch.
//
// Every sub-volume keeps its own context (fields, FP32 work, CG state and
// captured iteration chunk).  The batch driver starts each volume's
// mixed-precision solve (set-up kernels on the volume's stream), then builds
// one parent CUDA graph with, per volume, a WHILE conditional node whose
// body is the volume's iteration-chunk graph followed by a one-thread kernel
// that re-arms the condition while the volume's `done` flag is clear.  One
// cudaGraphLaunch therefore runs every volume to convergence, the volumes'
// kernels side by side on the GPU, and a converged volume stops launching
// anything.  The loop is bounded: after max_it + 2 rounds (each round is at
// least one iteration) the volume is marked as having hit the iteration cap.
// No counterpart in the reference, which solves one domain per MPI job.
#include <cstring>
#include <mutex>
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
  int* rounds = nullptr;  // device: rounds run per volume
  int nvol = 0;
};
BatchCache g_batch;
// Batch calls from several host threads take turns: the cached parent graph
// and its round counters are shared by every call.
std::mutex g_batch_mu;

}  // namespace

extern "C" int sbm_batch_solve_ops(sbm_ctx** ctxs, const int* ops, const int* bcx0,
                                   const int* bcx1, const double* scales, int n, double tol,
                                   int max_it, int precond, int* iters, double* final_res,
                                   int* status, float* ms_total) {
  if (!ctxs || !ops || !bcx0 || !bcx1 || !scales || n < 1 || max_it < 1 || !(tol >= 0.0))
    return SBM_ERR_ARG;
  if (precond != SBM_PC_NONE && precond != SBM_PC_JACOBI && precond != SBM_PC_LEARNED)
    return SBM_ERR_ARG;
  for (int v = 0; v < n; ++v)
    if (!ctxs[v] || (ops[v] != SBM_OP_GENERIC && ops[v] != SBM_OP_GENERIC_DIAG) ||
        (bcx0[v] != SBM_BC_COPY && bcx0[v] != SBM_BC_ZERO) ||
        (bcx1[v] != SBM_BC_COPY && bcx1[v] != SBM_BC_ZERO))
      return SBM_ERR_ARG;
  std::lock_guard<std::mutex> batch_lock(g_batch_mu);
  std::vector<SolveSpec> specs(n);
  std::vector<cudaGraph_t> graphs(n);
  std::vector<int> vnodes((size_t)n, 0);
  cudaStream_t bs = ctxs[0]->stream;  // the batch runs on the first volume's stream
  // events and the pinned state copies, released on every return path
  struct Scratch {
    cudaEvent_t t0 = nullptr, t1 = nullptr, ev = nullptr;
    CgState* h = nullptr;
    ~Scratch() {
      if (t0) cudaEventDestroy(t0);
      if (t1) cudaEventDestroy(t1);
      if (ev) cudaEventDestroy(ev);
      if (h) cudaFreeHost(h);
    }
  } sc;
  cudaEvent_t& t0 = sc.t0;
  cudaEvent_t& t1 = sc.t1;
  SBM_CUDA_TRY(cudaEventCreate(&t0));
  SBM_CUDA_TRY(cudaEventCreate(&t1));
  SBM_CUDA_TRY(cudaEventRecord(t0, bs));
  std::string key;
  char kbuf[32];
  int nodes_total = 0;
  for (int v = 0; v < n; ++v) {
    sbm_ctx* c = ctxs[v];
    SBM_CUDA_TRY(cudaStreamWaitEvent(c->stream, t0, 0));
    int rc = generic_spec(c, ops[v], bcx0[v], bcx1[v], scales[v], tol, max_it, SBM_STOP_REL_RES,
                          SBM_PREC_MIXED, precond, &specs[v]);
    if (rc) return rc;
    cudaGraphExec_t ex = nullptr;
    int nodes = 0;
    rc = mixed_begin(c, specs[v], &ex, &graphs[v], &nodes);
    if (rc) return rc;
    nodes_total += nodes;
    vnodes[v] = nodes;
    char buf[48];
    snprintf(buf, sizeof(buf), "%p,", (void*)graphs[v]);
    key += buf;
    // the batch stream waits for this volume's set-up
    cudaEvent_t e = c->evq[0];
    SBM_CUDA_TRY(cudaEventRecord(e, c->stream));
    SBM_CUDA_TRY(cudaStreamWaitEvent(bs, e, 0));
  }
  snprintf(kbuf, sizeof(kbuf), "cap%d", max_it);
  key += kbuf;
  if (key != g_batch.key) {
    if (g_batch.exec) cudaGraphExecDestroy(g_batch.exec);
    if (g_batch.parent) cudaGraphDestroy(g_batch.parent);
    if (g_batch.rounds) cudaFree(g_batch.rounds);
    g_batch = BatchCache();
    SBM_CUDA_TRY(cudaMalloc(&g_batch.rounds, sizeof(int) * n));
    g_batch.nvol = n;
    SBM_CUDA_TRY(cudaGraphCreate(&g_batch.parent, 0));
    const int cap = max_it + 2;
    for (int v = 0; v < n; ++v) {
      cudaGraphConditionalHandle h;
      SBM_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, g_batch.parent, 0,
                                                    cudaGraphCondAssignDefault));
      cudaGraphNode_t first, loop, child, last;
      int rc = add_graph_loop_node(g_batch.parent, nullptr, h, ctxs[v]->st, g_batch.rounds + v,
                                   cap, 1, &first);
      if (rc) return rc;
      cudaGraphNodeParams cp{};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = h;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      SBM_CUDA_TRY(cudaGraphAddNode(&loop, g_batch.parent, &first, nullptr, 1, &cp));
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      SBM_CUDA_TRY(cudaGraphAddChildGraphNode(&child, body, nullptr, 0, graphs[v]));
      if ((rc = add_graph_loop_node(body, &child, h, ctxs[v]->st, g_batch.rounds + v, cap, 0,
                                    &last)))
        return rc;
    }
    SBM_CUDA_TRY(cudaGraphInstantiate(&g_batch.exec, g_batch.parent, 0));
    g_batch.key = key;
    g_batch.nodes = nodes_total;
  }
  // one launch runs every volume to convergence; then all states and round
  // counts come back in one go
  CgState*& h = sc.h;
  SBM_CUDA_TRY(cudaMallocHost(&h, sizeof(CgState) * n));
  std::vector<int> rounds((size_t)n, 0);
  cudaEvent_t& ev = sc.ev;
  SBM_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  int rc = SBM_OK;
  SBM_CUDA_TRY(cudaGraphLaunch(g_batch.exec, bs));
  for (int v = 0; v < n; ++v)
    SBM_CUDA_TRY(cudaMemcpyAsync(&h[v], ctxs[v]->st, sizeof(CgState), cudaMemcpyDeviceToHost, bs));
  SBM_CUDA_TRY(cudaMemcpyAsync(rounds.data(), g_batch.rounds, sizeof(int) * n,
                               cudaMemcpyDeviceToHost, bs));
  SBM_CUDA_TRY(cudaEventRecord(ev, bs));
  if (cudaEventSynchronize(ev) != cudaSuccess) rc = SBM_ERR_CUDA;
  if (rc == SBM_OK) {
    int64_t launched = 0;
    for (int v = 0; v < n; ++v) launched += (int64_t)rounds[v] * (vnodes[v] + 1) + 1;
    SBM_LAUNCHED(launched);
  }
  if (rc == SBM_OK) {
    for (int v = 0; v < n && rc == SBM_OK; ++v) {
      sbm_ctx* c = ctxs[v];
      SBM_CUDA_TRY(cudaStreamWaitEvent(c->stream, ev, 0));
      SolveResult res{};
      rc = mixed_end(c, specs[v], h[v], &res);
      if (rc) break;
      // same post-condition as a single solve: Dirichlet faces keep their
      // data, the other ghosts copy the edge
      if ((rc = ghost_after_solve(c, specs[v].x, bcx0[v], bcx1[v]))) break;
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
  return rc;
}

extern "C" int sbm_batch_solve(sbm_ctx** ctxs, int n, int bc_x0, int bc_x1, double scale,
                               double tol, int max_it, int precond, int* iters, double* final_res,
                               int* status, float* ms_total) {
  if (n < 1) return SBM_ERR_ARG;
  std::vector<int> ops((size_t)n, SBM_OP_GENERIC), b0((size_t)n, bc_x0), b1((size_t)n, bc_x1);
  std::vector<double> sc((size_t)n, scale);
  return sbm_batch_solve_ops(ctxs, ops.data(), b0.data(), b1.data(), sc.data(), n, tol, max_it,
                             precond, iters, final_res, status, ms_total);
}
