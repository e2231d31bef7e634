// SQUANDER's ADAM decomposition engine advanced one cost evaluation at a time, shared by
// the batched decomposition kernel (decompose.cu: one CTA per target, the evaluation in
// shared memory) and the graph-driven single-target loop (loop.cu: the evaluation by the
// tile kernels, this state in global memory).
//
// Restated from Optimization_Interface::solve_layer_optimization_problem_ADAM
// (optimization_engines/ADAM.cpp:44-330) with its Adam optimizer (common/Adam.cpp: beta1
// 0.68, beta2 0.8, epsilon 1e-4; reset :70-100, update :138-270) and randomize_parameters
// (decomposition/Optimization_Interface.cpp:576-607: 30% of the parameters moved by
// U(-2 pi, 2 pi) * sqrt(f) around the best point).  The scalar bookkeeping (AdamRun) is
// replicated in every thread of the CTA; thread 0 draws the random numbers from the
// target's splitmix64 stream.  Adam's bias-correction powers advance once per parameter in
// parameter order, as in the reference; pw1/pw2 hold beta^(i + 1).
//
// Every routine is called by all threads of one CTA (blockDim.x a multiple of 32, at most
// kTileMaxThreads).
#pragma once
#include <cfloat>

#include "tile.cuh"

namespace sqg {

__device__ __forceinline__ unsigned long long splitmix_step(unsigned long long& s) {
  s += 0x9E3779B97F4A7C15ULL;
  unsigned long long z = s;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double splitmix_u01(unsigned long long& s) {
  return (double)(splitmix_step(s) >> 11) * (1.0 / 9007199254740992.0);
}

struct AdamConfig {
  int P;
  double tol;
  double eta;  // learning rate at the start of every engine call
  int adaptive_eta, shift_max;
  long long rand_thr;  // randomization_threshold: sub-iterations without progress
};

// Scalar state of one engine call.
struct AdamRun {
  double eta, beta1_t, beta2_t, f0_mean, dec_test, f0_prev, hold, cur_min;
  long long sub_iter;
  int f0_idx, dec_idx, status, shift_cnt;
};

// Vectors of one engine call: xt is the point being evaluated and g its gradient; f0_vec
// has 100 entries, dec_vec 20, red 2 * kTileMaxWarps (reduction scratch).
struct AdamVecs {
  double *xt, *g, *best, *mom, *var, *pw1, *pw2, *f0_vec;
  int* dec_vec;
  double* red;
};

constexpr double kAdamBeta1 = 0.68, kAdamBeta2 = 0.8, kAdamEps = 1e-4;

// beta^(i + 1) for i < P by repeated multiplication (thread 0; visible after the next barrier).
__device__ __forceinline__ void adam_powers(const AdamVecs& v, int P) {
  if (threadIdx.x == 0) {
    double t1 = 1.0, t2 = 1.0;
    for (int i = 0; i < P; i++) {
      t1 = t1 * kAdamBeta1;
      t2 = t2 * kAdamBeta2;
      v.pw1[i] = t1;
      v.pw2[i] = t2;
    }
  }
}

// Adam::reset: zero moments, the cost window and the decreasing-test window.
__device__ __forceinline__ void adam_reset_vectors(const AdamVecs& v, int P) {
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    v.mom[i] = 0.0;
    v.var[i] = 0.0;
  }
  for (int i = threadIdx.x; i < 100; i += blockDim.x) v.f0_vec[i] = 0.0;
  for (int i = threadIdx.x; i < 20; i += blockDim.x) v.dec_vec[i] = -1;
}

__device__ __forceinline__ void adam_reset_scalars(AdamRun& s) {
  s.beta1_t = 1.0;
  s.beta2_t = 1.0;
  s.f0_mean = 0.0;
  s.f0_idx = 0;
  s.dec_idx = 0;
  s.dec_test = -1.0;
  s.f0_prev = DBL_MAX;
}

// Start of an engine call at v.xt with the running minimum cur_min (carried across the
// outer iterations, as Decomposition_Base keeps current_minimum).  Ends with a barrier.
__device__ __forceinline__ void adam_begin(AdamRun& s, const AdamConfig& c, const AdamVecs& v, double cur_min) {
  adam_reset_scalars(s);
  s.eta = c.eta;
  s.hold = cur_min;
  s.cur_min = cur_min;
  s.sub_iter = 0;
  s.status = 0;
  s.shift_cnt = 0;
  adam_reset_vectors(v, c.P);
  for (int i = threadIdx.x; i < c.P; i += blockDim.x) v.best[i] = v.xt[i];
  __syncthreads();
}

// One pass of the engine loop after the cost f0 and gradient v.g at v.xt are known: the
// hold and learning-rate bookkeeping, the best point, the stop test, then either a
// randomisation of v.xt around the best point or one Adam step of v.xt.  Returns true when
// the engine call stops (tolerance reached or the randomisation limit passed) before any
// change of v.xt.  Ends with a barrier.
__device__ __forceinline__ bool adam_after_eval(AdamRun& s, const AdamConfig& c, const AdamVecs& v, double f0,
                                                unsigned long long& rng) {
  const int P = c.P;
  const double kPi = 3.14159265358979323846;
  if (s.sub_iter == 1) {
    s.hold = f0;
    if (c.adaptive_eta) s.eta = s.eta > 1e-3 ? s.eta : 1e-3;
  }
  if (s.hold * 0.95 > f0 || (s.hold * 0.97 > f0 && f0 < 1e-3) || (s.hold * 0.99 > f0 && f0 < 1e-4)) {
    s.sub_iter = 0;
    s.hold = f0;
  }
  if (s.cur_min > f0) {
    s.cur_min = f0;
    for (int i = threadIdx.x; i < P; i += blockDim.x) v.best[i] = v.xt[i];
    if (c.adaptive_eta) {  // the second clamp overwrites the first, as in the reference
      const double ne = 1e-3 * f0;
      s.eta = ne > 1e-6 ? ne : 1e-6;
      s.eta = ne < 1e-1 ? ne : 1e-1;
    }
  }
  if (f0 < c.tol || s.shift_cnt > c.shift_max) {
    __syncthreads();
    return true;
  }
  if (s.sub_iter > c.rand_thr || s.status != 0) {
    s.sub_iter = 0;
    s.shift_cnt++;
    s.hold = s.cur_min;
    __syncthreads();  // the best point is complete
    if (threadIdx.x == 0) {
      const double r = sqrt(f0);
      for (int j = 0; j < P; j++) {
        if (splitmix_u01(rng) <= 0.3)
          v.xt[j] = v.best[j] + (-2 * kPi + 4 * kPi * splitmix_u01(rng)) * r * 1.0;
        else
          v.xt[j] = v.best[j];
      }
    }
    adam_reset_scalars(s);
    adam_reset_vectors(v, P);
    s.status = 0;
    __syncthreads();
  } else {
    s.f0_mean = s.f0_mean + (f0 - v.f0_vec[s.f0_idx]) / 100;
    int dv = v.dec_vec[s.dec_idx];
    __syncthreads();  // every thread has read the entries rewritten below
    if (threadIdx.x == 0) v.f0_vec[s.f0_idx] = f0;
    s.f0_idx = (s.f0_idx + 1) % 100;
    if (f0 < s.f0_prev) {
      if (dv != 1) s.dec_test = s.dec_test + 2.0 / 20;
      dv = 1;
    } else {
      if (dv == 1) s.dec_test = s.dec_test - 2.0 / 20;
      dv = -1;
    }
    if (threadIdx.x == 0) v.dec_vec[s.dec_idx] = dv;
    s.dec_idx = (s.dec_idx + 1) % 20;
    s.f0_prev = f0;
    double red[2] = {0.0, 0.0};
    __syncthreads();  // the new window entry is visible below
    for (int i = threadIdx.x; i < 100; i += blockDim.x) {
      const double d = v.f0_vec[i] - s.f0_mean;
      red[0] = fma(d, d, red[0]);
    }
    for (int i = threadIdx.x; i < P; i += blockDim.x) red[1] += v.var[i];
    block_allsum_n(red, v.red);
    const double var_f0 = sqrt(red[0]) / 100, grad_var = red[1];
    const double eps = (grad_var < kAdamEps && s.dec_test > 0.7) ? kAdamEps / 100 : kAdamEps;
    const double b1 = kAdamBeta1, b2 = kAdamBeta2;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
      const double gi = v.g[i];
      const double m = b1 * v.mom[i] + (1 - b1) * gi;
      const double w = b2 * v.var[i] + (1 - b2) * gi * gi;
      v.mom[i] = m;
      v.var[i] = w;
      const double mh = m / (1 - s.beta1_t * v.pw1[i]);
      const double vh = w / (1 - s.beta2_t * v.pw2[i]);
      v.xt[i] = v.xt[i] - s.eta * mh / (sqrt(vh) + eps);
    }
    s.beta1_t = s.beta1_t * v.pw1[P - 1];
    s.beta2_t = s.beta2_t * v.pw2[P - 1];
    s.status = (fabs(s.f0_mean - f0) < 1e-6 && s.dec_test <= 0.7 && var_f0 / s.f0_mean < 1e-6) ? 1 : 0;
    __syncthreads();
  }
  s.sub_iter++;
  return false;
}

}  // namespace sqg
