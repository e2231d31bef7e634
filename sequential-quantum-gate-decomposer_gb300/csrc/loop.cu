// Graph-driven single-target decompositions: SQUANDER's ADAM engine or its BFGS driver for
// one target of any register size the gradient supports, run as ONE CUDA graph launch with no
// host round trip between evaluations.
//
// The graph holds a conditional WHILE node whose body is
//   [cost + gradient at the parameters x: the engine's own kernels, sqg_cost_grad]
//   -> [one CTA: the optimizer's work up to the next point to evaluate]
// and the controller clears the loop condition once the decomposition is over.  The optimizer
// state lives in the workspace between body executions.  Every body execution is one
// evaluation, and each engine call / BFGS run has a bounded evaluation budget, so the loop ends
// after at most (budget x calls) executions whatever the costs are.
//
// Reference loops: Optimization_Interface::solve_layer_optimization_problem_ADAM
// (optimization_engines/ADAM.cpp:44-330), the optimizer N_Qubit_Decomposition_custom picks above
// five qubits (N_Qubit_Decomposition_custom.cpp:59-76), and the BFGS decomposition
// (optimization_engines/BFGS.cpp:42-152 with common/BFGS_Powell.cpp:70-396); in both every
// iteration is a host call of the cost function and its gradient.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "../../include/sqg.h"
#include "adam.cuh"
#include "bfgs.cuh"
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

// ---- BFGS -------------------------------------------------------------------------------
// The BFGS decomposition driver of k_decompose (decompose.cu: dec_bfgs and the restart loop of
// k_decompose<kBfgs>) as a state machine that advances one evaluation at a time.

enum { kPhaseFirst = 0, kPhaseSearch = 1 };

struct BfgsState {
  double f, fprev, norm_Z, best;
  double step, f_low, f_high, s_high, s_low, s_best, f_best, dg, dg_best, dg_high;
  unsigned long long ctr;
  int phase, it, run, calls, iters, loop, outer;
};

struct BfgsLoopArgs {
  int P, max_calls, max_outer, loops, early_stop;
  double tol;
  BfgsState* st;
  double* cost;  // cost at v.x from the body's evaluation (gradient in v.g)
  BfgsVecs v;    // redd / scratch are set by each kernel to its shared memory
  double *bestx, *guess;
  double* x;  // start point on entry, best point on exit
  double* cost_out;
  int* calls_out;
  int* iters_out;
};

constexpr int kBfgsVectors = 19;  // the 17 vectors of BfgsVecs, bestx and guess

struct BfgsLayout {
  size_t st, cost, vec[kBfgsVectors], Z, eval, end;
};

BfgsLayout bfgs_layout(const sqg_circuit* c, int cols) {
  BfgsLayout l = {};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t r = off;
    off += (bytes + 255) / 256 * 256;
    return r;
  };
  l.st = take(sizeof(BfgsState));
  l.cost = take(sizeof(double));
  for (size_t& v : l.vec) v = take(sizeof(double) * (size_t)c->P);
  l.Z = take(sizeof(double) * (size_t)c->P * c->P);
  l.eval = take(sqg_cost_grad_workspace_bytes(c, 1, cols, 1));
  l.end = off;
  return l;
}

// Threads of the BFGS controller: as k_decompose up to 128 parameters (so that its reductions
// run in the same order), 256 above.
int bfgs_threads(int P) { return P <= 128 ? std::min(128, std::max(64, (P + 31) / 32 * 32)) : 256; }

// A BFGS run starts at guess with Z = I (BFGS_Powell::Optimize); its first evaluation is at x.
__device__ void bfgs_start_run(const BfgsLoopArgs& a, const BfgsVecs& v, BfgsState& s) {
  const int P = a.P;
  for (int i = threadIdx.x; i < P; i += blockDim.x) v.x[i] = a.guess[i];
  for (long long i = threadIdx.x; i < (long long)P * P; i += blockDim.x) v.Z[i] = (i % (P + 1)) == 0 ? 1.0 : 0.0;
  s.norm_Z = -1.0;
  s.run = 0;
  s.phase = kPhaseFirst;
  __syncthreads();
}

// End of a BFGS run with minimum f and final point v.x: the restart bookkeeping of
// k_decompose<kBfgs> (the best point, its perturbation by U[0, 2 pi)/100, iteration_loops runs
// per outer iteration).  Returns true when the decomposition is over.
__device__ bool bfgs_end_run(const BfgsLoopArgs& a, const BfgsVecs& v, BfgsState& s, double f) {
  const int P = a.P;
  for (int i = threadIdx.x; i < P; i += blockDim.x) a.guess[i] = v.x[i];
  if (f < s.best) {
    s.best = f;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
      a.bestx[i] = v.x[i];
      a.guess[i] = v.x[i] + u01(s.ctr + i) * kTwoPi / 100.0;
    }
    s.ctr += 0x100000001ULL * (unsigned long long)(P + 1);
  }
  __syncthreads();
  if (a.early_stop && s.best < a.tol) return true;
  if (++s.loop < a.loops) return false;
  s.loop = 0;
  for (int i = threadIdx.x; i < P; i += blockDim.x) a.guess[i] = a.bestx[i];
  __syncthreads();
  if (fabs(s.best) < a.tol) return true;
  return ++s.outer >= a.max_outer;
}

__device__ __forceinline__ BfgsVecs bfgs_vecs(const BfgsLoopArgs& a, double* redd, double* scratch) {
  BfgsVecs v = a.v;
  v.redd = redd;
  v.scratch = scratch;
  return v;
}

__global__ void __launch_bounds__(kLoopThreads) k_bfgs_loop_begin(BfgsLoopArgs a, unsigned long long seed) {
  __shared__ double redd[kTileMaxWarps * 8], scratch[kTileMaxWarps];
  const BfgsVecs v = bfgs_vecs(a, redd, scratch);
  for (int i = threadIdx.x; i < a.P; i += blockDim.x) a.guess[i] = a.x[i];
  __syncthreads();
  BfgsState s = {};
  s.best = INFINITY;
  s.ctr = seed * 0x2545F4914F6CDD1DULL;
  bfgs_start_run(a, v, s);
  if (threadIdx.x == 0) *a.st = s;
}

// Consumes the evaluation at v.x (cost, gradient v.g) and runs BFGS_Powell up to the next point
// to evaluate (written to v.x) or to the end of the decomposition (BFGS_Powell.cpp:70-192 and
// the line search of grad_descend.cpp:127-273, in the order of dec_bfgs).
__global__ void __launch_bounds__(kLoopThreads) k_bfgs_loop_step(BfgsLoopArgs a, cudaGraphConditionalHandle h) {
  __shared__ double redd[kTileMaxWarps * 8], scratch[kTileMaxWarps];
  const BfgsVecs v = bfgs_vecs(a, redd, scratch);
  const int P = a.P;
  BfgsState s = *a.st;
  const double f = *a.cost;
  __syncthreads();  // every thread holds the state before thread 0 rewrites it
  s.calls++;
  s.run++;
  s.f = f;
  bool run_over = false, ls_end = false, direction = false, done = false;
  if (s.phase == kPhaseFirst) {
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
      v.cs[i] = 1.0;
      v.ztg[i] = v.g[i];
      v.zs[i] = v.g[i];
    }
    __syncthreads();
    if (a.early_stop && f < a.tol) {
      run_over = true;
    } else {
      s.fprev = fabs(f + f + 1.0);
      direction = true;
    }
  } else if (a.early_stop && f < a.tol) {
    run_over = true;
  } else {  // line-search evaluation at s.step
    const double dgc = dot(v.d, v.g, P, v.scratch);
    if (f < s.f_best || fabs(dgc) < s.dg_best) {
      s.s_best = s.step;
      s.f_best = f;
      s.dg_best = fabs(dgc);
      for (int i = threadIdx.x; i < P; i += blockDim.x) v.gbest[i] = v.g[i];
      __syncthreads();
    }
    bool brk = s.run == a.max_calls;
    if (!brk) {
      if (f < s.f_low + s.step * 0.1 * s.dg) {
        if (dgc >= s.dg * 0.7) {
          brk = true;
        } else {
          s.s_low = s.step;
          s.f_low = f;
        }
      } else {
        s.s_high = s.step;
        s.f_high = f;
        s.dg_high = dgc;
      }
    }
    if (!brk) {
      if (s.it == 0 || s.s_low > 0.0) {
        const double dlf = (s.f_high - s.f_low) / (s.s_high - s.s_low) * 2.0 - s.dg_high;
        double scale = -dlf * 0.5 / (s.dg_high - dlf);
        scale = fmax(0.1, scale);
        s.step = s.s_low + scale * (s.s_high - s.s_low);
      } else {
        s.step = s.step * 0.1;
        if (s.step < kNumPrecision) brk = true;
      }
    }
    if (!brk && ++s.it >= 50) brk = true;
    ls_end = brk;
  }
  if (ls_end) {
    if (s.step != s.s_best) {
      s.step = s.s_best;
      s.f = s.f_best;
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        v.g[i] = v.gbest[i];
        v.x[i] = v.x0[i] + s.step * v.d[i];
      }
      __syncthreads();
    }
    if (s.step == 0.0) {
      run_over = true;
    } else {
      s.norm_Z = bfgs_update(P, v, s.norm_Z, ZMem{});
      direction = true;
    }
  }
  bool search = !ls_end && !run_over && !direction;  // the line search goes on at s.step
  if (direction) {
    double dg, max_step, gn;
    bfgs_direction(P, v, dg, max_step, gn, ZMem{});
    if (gn <= 1e-19 * 1e-19 || dg >= 0.0 || s.f >= s.fprev) {
      run_over = true;
    } else {
      s.fprev = s.f;
      if (s.run >= a.max_calls) {
        run_over = true;
      } else {
        s.iters++;
        for (int i = threadIdx.x; i < P; i += blockDim.x) {
          v.x0[i] = v.x[i];
          v.g0[i] = v.g[i];
          v.gbest[i] = v.g[i];
        }
        __syncthreads();
        s.dg = dg;
        s.step = fmin(1.0, max_step);
        s.f_low = s.f_high = s.f_best = s.f;
        s.s_high = max_step;
        s.s_low = s.s_best = s.dg_high = 0.0;
        s.dg_best = fabs(dg);
        s.it = 0;
        s.phase = kPhaseSearch;
        search = true;
      }
    }
  }
  if (run_over) {
    if (bfgs_end_run(a, v, s, s.f))
      done = true;
    else
      bfgs_start_run(a, v, s);  // the next evaluation is the new run's first, at v.x
  } else if (search) {
    for (int i = threadIdx.x; i < P; i += blockDim.x) v.x[i] = v.x0[i] + s.step * v.d[i];
  }
  // defensive cap: every run has at most max_calls evaluations
  if (!done && (long long)s.calls >= (long long)a.max_calls * a.loops * a.max_outer + 1) done = true;
  if (done)
    for (int i = threadIdx.x; i < P; i += blockDim.x) a.x[i] = a.bestx[i];
  if (threadIdx.x == 0) {
    *a.st = s;
    if (done) {
      *a.cost_out = s.best;
      *a.calls_out = s.calls;
      if (a.iters_out) *a.iters_out = s.iters;
      cudaGraphSetConditional(h, 0);
    }
  }
}

// Builds the graph [while (cond) { cost + gradient at x_eval; step }], runs begin on the
// stream, launches the graph after it and releases the graph (it finishes on its own).
template <class Step, class Begin>
int run_loop_graph(const sqg_circuit* c, const void* target, int cols, int trace_offset, int cost_variant,
                   const double* x_eval, double* cost_eval, double* g_eval, char* eval_ws, size_t eval_bytes,
                   Step step, Begin begin, cudaStream_t stream) {
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
    st = sqg_cost_grad(c, x_eval, 1, target, cols, 0, trace_offset, cost_variant, cost_eval, g_eval, 0, eval_ws,
                       eval_bytes, cap);
    if (st == SQG_OK) {
      step(cap, handle);
      e = cudaGetLastError();
      if (e != cudaSuccess) st = cuda_fail(e, "decomposition loop step kernel");
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
    begin(stream);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaGraphLaunch(exec, stream);
    if (e != cudaSuccess) st = cuda_fail(e, "launching the decomposition graph");
  }
  // an executable graph destroyed while in flight is released when it completes
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (cap) cudaStreamDestroy(cap);
  return st;
}

int check_loop_args(const sqg_circuit* c, const void* target, const double* x, const double* cost, const int* count,
                    int cols, int trace_offset, int cost_variant) {
  if (!c || !target || !x || !cost || !count || cols <= 0 || cols > c->N)
    return set_error(SQG_ERR_INVALID_ARGUMENT, "bad circuit, target or outputs");
  if (c->P == 0) return set_error(SQG_ERR_INVALID_ARGUMENT, "the circuit has no free parameters");
  if (c->n > 12) return set_error(SQG_ERR_UNSUPPORTED, "gradient supports qbit_num <= 12");
  if (cost_variant != SQG_FROBENIUS_NORM && cost_variant != SQG_HILBERT_SCHMIDT_TEST && cost_variant != SQG_INFIDELITY)
    return set_error(SQG_ERR_UNSUPPORTED, "cost function variant not implemented by the engine");
  const int off = cost_variant == SQG_FROBENIUS_NORM ? trace_offset : 0;
  if (off < 0 || off + cols > c->N) return set_error(SQG_ERR_INVALID_ARGUMENT, "trace offset out of range");
  return SQG_OK;
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
  int st = check_loop_args(c, target, x, cost, evals, cols, trace_offset, cost_variant);
  if (st) return st;
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
  return run_loop_graph(
      c, target, cols, trace_offset, cost_variant, a.xt, a.cost, a.g, ws + l.eval, l.end - l.eval,
      [&](cudaStream_t s, cudaGraphConditionalHandle h) { k_adam_loop_step<<<1, kLoopThreads, 0, s>>>(a, h); },
      [&](cudaStream_t s) { k_adam_loop_begin<<<1, kLoopThreads, 0, s>>>(a, current_minimum, seed); },
      (cudaStream_t)stream);
}

size_t sqg_bfgs_loop_workspace_bytes(const sqg_circuit* c, int cols) {
  if (!c || cols <= 0 || c->P <= 0) return 0;
  return bfgs_layout(c, cols).end;
}

int sqg_decompose_bfgs_loop(const sqg_circuit* c, const void* target, int cols, int trace_offset, int cost_variant,
                            double* x, double* cost, int* calls, int* iters, double tolerance, int max_calls,
                            int max_outer, int iteration_loops, int stop_at_tolerance, unsigned long long seed,
                            void* workspace, size_t ws_bytes, void* stream) {
  int st = check_loop_args(c, target, x, cost, calls, cols, trace_offset, cost_variant);
  if (st) return st;
  if (max_calls < 1 || max_outer < 1 || iteration_loops < 1)
    return set_error(SQG_ERR_INVALID_ARGUMENT, "iteration limits must be positive");
  const BfgsLayout l = bfgs_layout(c, cols);
  if (!workspace || ws_bytes < l.end || ((size_t)workspace & 255))
    return set_error(SQG_ERR_WORKSPACE, "workspace too small or not 256-byte aligned: need " + std::to_string(l.end));
  char* ws = (char*)workspace;
  BfgsLoopArgs a = {};
  a.P = c->P;
  a.max_calls = max_calls;
  a.max_outer = max_outer;
  a.loops = iteration_loops;
  a.early_stop = stop_at_tolerance ? 1 : 0;
  a.tol = tolerance;
  a.st = (BfgsState*)(ws + l.st);
  a.cost = (double*)(ws + l.cost);
  double** vecs[kBfgsVectors] = {&a.v.x, &a.v.x0, &a.v.g, &a.v.g0, &a.v.gbest, &a.v.d, &a.v.delta,
                                 &a.v.gamma, &a.v.v, &a.v.vp, &a.v.cs, &a.v.ztg, &a.v.zs, &a.v.S,
                                 &a.v.sdv, &a.v.nz, &a.v.gtz, &a.bestx, &a.guess};
  for (int k = 0; k < kBfgsVectors; k++) *vecs[k] = (double*)(ws + l.vec[k]);
  a.v.Z = (double*)(ws + l.Z);
  a.x = x;
  a.cost_out = cost;
  a.calls_out = calls;
  a.iters_out = iters;
  const int threads = bfgs_threads(c->P);
  return run_loop_graph(
      c, target, cols, trace_offset, cost_variant, a.v.x, a.cost, a.v.g, ws + l.eval, l.end - l.eval,
      [&](cudaStream_t s, cudaGraphConditionalHandle h) { k_bfgs_loop_step<<<1, threads, 0, s>>>(a, h); },
      [&](cudaStream_t s) { k_bfgs_loop_begin<<<1, threads, 0, s>>>(a, seed); }, (cudaStream_t)stream);
}

}  // extern "C"
