// Graph-driven single-target decomposition: SQUANDER's ADAM engine for one target of any
// register size the gradient supports, run as ONE CUDA graph launch with no host round
// trip between evaluations.
//
// The graph holds a conditional WHILE node whose body is
//   [cost + gradient of the parameters xt: the engine's own kernels, sqg_cost_grad]
//   -> [k_adam_loop_step: one pass of the ADAM engine loop on one CTA]
// and k_adam_loop_step clears the loop condition once the decomposition is over.  The
// engine state (adam.cuh) lives in the workspace between body executions.  Each body
// execution either advances the evaluation count of the current engine call (at most
// max_iters) or ends that call (at most max_outer), so the loop ends after at most
// max_iters * max_outer executions whatever the costs are.
//
// Reference loop: Optimization_Interface::solve_layer_optimization_problem_ADAM
// (optimization_engines/ADAM.cpp:44-330), the optimizer N_Qubit_Decomposition_custom picks
// above five qubits (N_Qubit_Decomposition_custom.cpp:59-76), whose every iteration there
// is a host call of the cost function and its gradient.
#include <cuda_runtime.h>

#include <string>

#include "../../include/sqg.h"
#include "adam.cuh"
#include "handle.h"

using namespace sqg;

namespace {

constexpr int kLoopThreads = 256;

struct LoopState {
  AdamRun run;
  unsigned long long rng;
  int it, outer, evals, shifts;
};

struct LoopArgs {
  AdamConfig cfg;
  int max_iters, max_outer;
  LoopState* st;
  double *xt, *g, *best, *mom, *var, *pw1, *pw2, *f0_vec, *cost;
  int* dec_vec;
  double* x;  // start point on entry, best point on exit
  double* cost_out;
  int* evals_out;
  int* shifts_out;
};

// Workspace layout: state, cost, seven P-vectors, the two windows, then the scratch of
// sqg_cost_grad; every part on a 256-byte boundary.
struct LoopLayout {
  size_t st, cost, vec[7], f0, dec, eval, end;
};

LoopLayout loop_layout(const sqg_circuit* c, int cols) {
  LoopLayout l = {};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t r = off;
    off += (bytes + 255) / 256 * 256;
    return r;
  };
  l.st = take(sizeof(LoopState));
  l.cost = take(sizeof(double));
  for (size_t& v : l.vec) v = take(sizeof(double) * (size_t)c->P);
  l.f0 = take(sizeof(double) * 100);
  l.dec = take(sizeof(int) * 20);
  l.eval = take(sqg_cost_grad_workspace_bytes(c, 1, cols, 1));
  l.end = off;
  return l;
}

__device__ __forceinline__ AdamVecs loop_vecs(const LoopArgs& a, double* red) {
  return AdamVecs{a.xt, a.g, a.best, a.mom, a.var, a.pw1, a.pw2, a.f0_vec, a.dec_vec, red};
}

// Engine state for the first call, from the start point a.x.
__global__ void __launch_bounds__(kLoopThreads) k_adam_loop_begin(LoopArgs a, double current_minimum,
                                                                  unsigned long long seed) {
  __shared__ double red[2 * kTileMaxWarps];
  const AdamVecs v = loop_vecs(a, red);
  for (int i = threadIdx.x; i < a.cfg.P; i += blockDim.x) v.xt[i] = a.x[i];
  adam_powers(v, a.cfg.P);
  __syncthreads();
  AdamRun s;
  adam_begin(s, a.cfg, v, current_minimum);
  if (threadIdx.x == 0) {
    a.st->run = s;
    a.st->rng = seed;
    a.st->it = 0;
    a.st->outer = 0;
    a.st->evals = 0;
    a.st->shifts = 0;
  }
}

// One pass of the engine loop after the evaluation of the body; clears the loop
// condition when the decomposition is over and then writes the results.
__global__ void __launch_bounds__(kLoopThreads) k_adam_loop_step(LoopArgs a, cudaGraphConditionalHandle h) {
  __shared__ double red[2 * kTileMaxWarps];
  const AdamVecs v = loop_vecs(a, red);
  AdamRun s = a.st->run;
  unsigned long long rng = a.st->rng;
  int it = a.st->it + 1, outer = a.st->outer, evals = a.st->evals + 1, shifts = a.st->shifts;
  const double f0 = *a.cost;
  __syncthreads();  // every thread holds the state before thread 0 rewrites it
  bool stop = adam_after_eval(s, a.cfg, v, f0, rng);
  if (!stop && it >= a.max_iters) stop = true;
  bool done = false;
  if (stop) {
    outer++;
    shifts += s.shift_cnt;
    if (fabs(s.cur_min) < a.cfg.tol || outer >= a.max_outer) {
      done = true;
    } else {  // the next engine call starts at the best point with the running minimum
      for (int i = threadIdx.x; i < a.cfg.P; i += blockDim.x) v.xt[i] = v.best[i];
      __syncthreads();
      adam_begin(s, a.cfg, v, s.cur_min);
      it = 0;
    }
  }
  if (done)
    for (int i = threadIdx.x; i < a.cfg.P; i += blockDim.x) a.x[i] = v.best[i];
  if (threadIdx.x == 0) {
    a.st->run = s;
    a.st->rng = rng;
    a.st->it = it;
    a.st->outer = outer;
    a.st->evals = evals;
    a.st->shifts = shifts;
    if (done) {
      *a.cost_out = s.cur_min;
      *a.evals_out = evals;
      if (a.shifts_out) *a.shifts_out = shifts;
      cudaGraphSetConditional(h, 0);
    }
  }
}

int cuda_fail(cudaError_t e, const char* where) {
  return set_error(SQG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

}  // namespace

extern "C" {

size_t sqg_adam_loop_workspace_bytes(const sqg_circuit* c, int cols) {
  if (!c || cols <= 0 || c->P <= 0) return 0;
  return loop_layout(c, cols).end;
}

int sqg_decompose_adam_loop(const sqg_circuit* c, const void* target, int cols, int trace_offset, int cost_variant,
                            double* x, double* cost, int* evals, int* shifts, double tolerance, int max_iters,
                            double eta, int adaptive_eta, int random_shift_count_max,
                            long long randomization_threshold, int max_outer, double current_minimum,
                            unsigned long long seed, void* workspace, size_t ws_bytes, void* stream) {
  if (!c || !target || !x || !cost || !evals || cols <= 0 || cols > c->N)
    return set_error(SQG_ERR_INVALID_ARGUMENT, "bad circuit, target or outputs");
  if (c->P == 0) return set_error(SQG_ERR_INVALID_ARGUMENT, "the circuit has no free parameters");
  if (c->n > 12) return set_error(SQG_ERR_UNSUPPORTED, "gradient supports qbit_num <= 12");
  if (cost_variant != SQG_FROBENIUS_NORM && cost_variant != SQG_HILBERT_SCHMIDT_TEST && cost_variant != SQG_INFIDELITY)
    return set_error(SQG_ERR_UNSUPPORTED, "cost function variant not implemented by the engine");
  const int off = cost_variant == SQG_FROBENIUS_NORM ? trace_offset : 0;
  if (off < 0 || off + cols > c->N) return set_error(SQG_ERR_INVALID_ARGUMENT, "trace offset out of range");
  if (max_iters < 1 || max_outer < 1 || random_shift_count_max < 0 || randomization_threshold < 0)
    return set_error(SQG_ERR_INVALID_ARGUMENT, "iteration limits must be positive");
  const LoopLayout l = loop_layout(c, cols);
  if (!workspace || ws_bytes < l.end || ((size_t)workspace & 255))
    return set_error(SQG_ERR_WORKSPACE, "workspace too small or not 256-byte aligned: need " + std::to_string(l.end));
  char* ws = (char*)workspace;
  LoopArgs a = {};
  a.cfg = AdamConfig{c->P, tolerance, eta, adaptive_eta ? 1 : 0, random_shift_count_max, randomization_threshold};
  a.max_iters = max_iters;
  a.max_outer = max_outer;
  a.st = (LoopState*)(ws + l.st);
  a.cost = (double*)(ws + l.cost);
  double** vecs[] = {&a.xt, &a.g, &a.best, &a.mom, &a.var, &a.pw1, &a.pw2};
  for (int k = 0; k < 7; k++) *vecs[k] = (double*)(ws + l.vec[k]);
  a.f0_vec = (double*)(ws + l.f0);
  a.dec_vec = (int*)(ws + l.dec);
  a.x = x;
  a.cost_out = cost;
  a.evals_out = evals;
  a.shifts_out = shifts;

  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cap = nullptr;
  int st = SQG_OK;
  cudaError_t e = cudaGraphCreate(&graph, 0);
  cudaGraphConditionalHandle handle = 0;
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault);
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = handle;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node = nullptr;
  if (e == cudaSuccess) e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
  if (e == cudaSuccess)
    e = cudaStreamBeginCaptureToGraph(cap, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) {
    st = cuda_fail(e, "building the decomposition graph");
  } else {
    st = sqg_cost_grad(c, a.xt, 1, target, cols, 0, trace_offset, cost_variant, a.cost, a.g, 0, ws + l.eval,
                       l.end - l.eval, cap);
    if (st == SQG_OK) {
      k_adam_loop_step<<<1, kLoopThreads, 0, cap>>>(a, handle);
      e = cudaGetLastError();
      if (e != cudaSuccess) st = cuda_fail(e, "k_adam_loop_step");
    }
    cudaGraph_t body = nullptr;
    e = cudaStreamEndCapture(cap, &body);
    if (st == SQG_OK && e != cudaSuccess) st = cuda_fail(e, "capturing the decomposition loop body");
  }
  if (st == SQG_OK) {
    e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) st = cuda_fail(e, "cudaGraphInstantiate");
  }
  if (st == SQG_OK) {
    k_adam_loop_begin<<<1, kLoopThreads, 0, (cudaStream_t)stream>>>(a, current_minimum, seed);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaGraphLaunch(exec, (cudaStream_t)stream);
    if (e != cudaSuccess) st = cuda_fail(e, "launching the decomposition graph");
  }
  // an executable graph destroyed while in flight is released when it completes
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (cap) cudaStreamDestroy(cap);
  return st;
}

}  // extern "C"
