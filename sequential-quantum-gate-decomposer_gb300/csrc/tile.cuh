// Shared-memory column-tile sweeps used by the evaluator kernels (engine.cu) and the
// batched decomposition kernel (decompose.cu).
//
// A tile holds tc vectors of length N (one column of the target each, column-major in
// shared memory).  Every routine is executed by all threads of the CTA; blockDim.x is a
// multiple of 32 and at most kTileMaxThreads.
#pragma once
#include "gates.cuh"

namespace sqg {

constexpr int kTileMaxThreads = 256;
constexpr int kTileMaxWarps = kTileMaxThreads / 32;

// Applies one gate to every vector of the tile; thread tid of nthr threads takes the
// amplitude pairs tid, tid + nthr, ...
__device__ __forceinline__ void tile_apply_by(double2* s, int N, int logN, int tc, const Gate& gt, const PairOp& op,
                                              int tid, int nthr) {
  const bool ctrl = gate_controlled(gt.type);
  const int lognp = ctrl ? logN - 2 : logN - 1;
  const int npairs = 1 << lognp;
  const int items = tc << lognp;
  const int step = 1 << gt.target;
  for (int it = tid; it < items; it += nthr) {
    int col = it >> lognp;
    int p = it & (npairs - 1);
    int i = ctrl ? pair_index2(p, gt.target, gt.control) : pair_index1(p, gt.target);
    double2* v = s + col * N;
    double2 x = v[i], y = v[i + step];
    apply_op(op, x, y);
    v[i] = x;
    v[i + step] = y;
  }
}

// Applies one gate to every vector of the tile (all threads of the CTA).
__device__ __forceinline__ void tile_apply(double2* s, int N, int logN, int tc, const Gate& gt, const PairOp& op) {
  tile_apply_by(s, N, logN, tc, gt, op, threadIdx.x, blockDim.x);
}

// Warp reduce-scatter of 8 doubles: afterwards lane l holds the warp total of value
// (l >> 2) & 7 (9 FP64 adds per lane instead of 40 for eight full butterflies).
__device__ __forceinline__ double warp_reduce_scatter8(double r[8]) {
  const int lane = threadIdx.x & 31;
  {
    const bool hi = lane & 16;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      double send = hi ? r[k] : r[k + 4];
      double keep = hi ? r[k + 4] : r[k];
      r[k] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
  }
  {
    const bool hi = lane & 8;
#pragma unroll
    for (int k = 0; k < 2; k++) {
      double send = hi ? r[k] : r[k + 2];
      double keep = hi ? r[k + 2] : r[k];
      r[k] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
  }
  {
    const bool hi = lane & 4;
    double send = hi ? r[0] : r[1];
    double keep = hi ? r[1] : r[0];
    r[0] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
  double v = r[0];
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  return v;
}

// Sum of v over the CTA, returned to every thread (fixed summation order, so all threads
// hold the identical value).  scratch: kTileMaxWarps doubles.
__device__ __forceinline__ double block_allsum(double v, double* scratch) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int nw = blockDim.x >> 5;
  if (nw == 1) return v;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < nw; w++) t += scratch[w];
  return t;
}

// Sums of K per-thread values over the CTA, returned to every thread in a fixed order.
// scratch: K * kTileMaxWarps doubles.
template <int K>
__device__ __forceinline__ void block_allsum_n(double (&v)[K], double* scratch) {
#pragma unroll
  for (int k = 0; k < K; k++)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  const int nw = blockDim.x >> 5, warp = threadIdx.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int k = 0; k < K; k++) scratch[k * kTileMaxWarps + warp] = v[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; k++) {
    double t = 0.0;
    for (int w = 0; w < nw; w++) t += scratch[k * kTileMaxWarps + w];
    v[k] = t;
  }
}

__device__ __forceinline__ double block_allmin(double v, double* scratch) {
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int nw = blockDim.x >> 5;
  if (nw == 1) return v;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = scratch[0];
  for (int w = 1; w < nw; w++) t = fmin(t, scratch[w]);
  return t;
}

// Complex trace partial sum_c s[c][v0 + c + offset] over the tile, returned to all threads.
__device__ __forceinline__ double2 tile_trace(const double2* s, int N, int tc, int v0, int offset, double* scratch) {
  double2 t = make_double2(0.0, 0.0);
  for (int c = threadIdx.x; c < tc; c += blockDim.x) {
    double2 v = s[c * N + v0 + c + offset];
    t.x += v.x;
    t.y += v.y;
  }
  t.x = block_allsum(t.x, scratch);
  t.y = block_allsum(t.y, scratch);
  return t;
}

// Reverse (adjoint) sweep over gates L-1..0.  On entry psi holds C u_j and lam holds
// e_{j + offset} for each vector of the tile.  For every parametric gate g the 2x2
// overlap R_ab = sum conj(lambda_a) psi_b (psi in front of the gate, lambda behind it)
// is reduced over the tile into tot[0..7] = (Re R00, Im R00, Re R01, Im R01, Re R10,
// Im R10, Re R11, Im R11) and sink(g, gate, tot) is called by every thread.
// Only the warps that own amplitude pairs of the gate take part in the reduction: the
// FP64 pipe is charged per warp instruction whatever the number of active lanes.
// redd: kTileMaxWarps * 8 doubles, tot: 8 doubles.  restore(g) is called at the start of
// each reverse step and may overwrite psi (checkpoints); it must contain its own barriers.
// stage_gates / stage_mats (kStage entries each, or null): shared-memory staging of the
// gate records and matrices when gates / gm are in global memory.
constexpr int kStage = 32;

template <class Sink, class Restore>
__device__ __forceinline__ void adjoint_sweep(double2* psi, double2* lam, int N, int logN, int tc, const Gate* gates,
                                              const GateMat* gm, const double2* sc, int L, double* redd, double* tot,
                                              Sink sink, Restore restore, Gate* stage_gates = nullptr,
                                              GateMat* stage_mats = nullptr) {
  const int nw = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool staged = stage_gates != nullptr;
  for (int g = L - 1; g >= 0; g--) {
    const int j = (L - 1 - g) % kStage;  // position of gate g in its staged chunk
    if (staged && j == 0) {
      __syncthreads();
      const int kn = min(kStage, g + 1);
      if ((int)threadIdx.x < kn) {
        stage_gates[threadIdx.x] = gates[g - threadIdx.x];
        stage_mats[threadIdx.x] = gm[g - threadIdx.x];
      }
      __syncthreads();
    }
    restore(g);
    Gate gt = staged ? stage_gates[j] : gates[g];
    PairOp op = make_op(gt.type, staged ? stage_mats[j] : gm[g], ORIENT_ADJ);
    const int np = gate_param_num(gt.type);
    if (np == 0) {
      tile_apply(psi, N, logN, tc, gt, op);
      tile_apply(lam, N, logN, tc, gt, op);
      __syncthreads();
      continue;
    }
    const bool ctrl = gate_controlled(gt.type);
    const int lognp = ctrl ? logN - 2 : logN - 1;
    const int npairs = 1 << lognp;
    const int items = tc << lognp;
    const int step = 1 << gt.target;
    double r[8];
#pragma unroll
    for (int k = 0; k < 8; k++) r[k] = 0.0;
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
      int col = it >> lognp;
      int p = it & (npairs - 1);
      int i = ctrl ? pair_index2(p, gt.target, gt.control) : pair_index1(p, gt.target);
      double2* ps = psi + col * N;
      double2* ls = lam + col * N;
      double2 x = ps[i], y = ps[i + step];
      apply_op(op, x, y);  // psi in front of gate g
      ps[i] = x;
      ps[i + step] = y;
      double2 lx = ls[i], ly = ls[i + step];
      r[0] = fma(lx.x, x.x, fma(lx.y, x.y, r[0]));
      r[1] = fma(lx.x, x.y, fma(-lx.y, x.x, r[1]));
      r[2] = fma(lx.x, y.x, fma(lx.y, y.y, r[2]));
      r[3] = fma(lx.x, y.y, fma(-lx.y, y.x, r[3]));
      r[4] = fma(ly.x, x.x, fma(ly.y, x.y, r[4]));
      r[5] = fma(ly.x, x.y, fma(-ly.y, x.x, r[5]));
      r[6] = fma(ly.x, y.x, fma(ly.y, y.y, r[6]));
      r[7] = fma(ly.x, y.y, fma(-ly.y, y.x, r[7]));
      apply_op(op, lx, ly);  // lambda in front of gate g
      ls[i] = lx;
      ls[i + step] = ly;
    }
    const int aw = min(nw, (items + 31) >> 5);  // warps holding pairs
    if (warp < aw) {
      double v = warp_reduce_scatter8(r);
      if ((lane & 3) == 0) {
        if (aw == 1)
          tot[lane >> 2] = v;
        else
          redd[warp * 8 + (lane >> 2)] = v;
      }
    }
    __syncthreads();
    if (aw > 1) {
      if (threadIdx.x < 8) {
        double t = 0.0;
        for (int w = 0; w < aw; w++) t += redd[w * 8 + threadIdx.x];
        tot[threadIdx.x] = t;
      }
      __syncthreads();
    }
    sink(g, gt, tot);
  }
}

// T = sum_ab D_ab R_ab for derivative parameter k of gate gt, R as laid out in tot.
__device__ __forceinline__ double2 contract_derivative(const Gate& gt, const double2* sc, int k, const double* R) {
  double2 D[4];
  deriv_kernel(gt.type, sc + gt.pstart, k, D);
  double tr = 0.0, ti = 0.0;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    double rr = R[2 * q], ri = R[2 * q + 1];
    tr = fma(D[q].x, rr, fma(-D[q].y, ri, tr));
    ti = fma(D[q].x, ri, fma(D[q].y, rr, ti));
  }
  return make_double2(tr, ti);
}

// Builds the gate matrices and per-parameter (sin, cos) of one parameter vector
// (threads over gates).  Same formulas as k_prep in engine.cu.
__device__ __forceinline__ void build_gate_mats(const Gate* gates, int L, const double* th, GateMat* gm, double2* sc) {
  for (int g = threadIdx.x; g < L; g += blockDim.x) {
    Gate gt = gates[g];
    GateMat m;
    m.u[0] = m.u[1] = m.u[2] = m.u[3] = make_double2(0.0, 0.0);
    if (gt.type == G_U3) {
      double st, ct, sp, cp, sl, cl;
      sincos(th[gt.pstart], &st, &ct);
      sincos(th[gt.pstart + 1], &sp, &cp);
      sincos(th[gt.pstart + 2], &sl, &cl);
      sc[gt.pstart] = make_double2(st, ct);
      sc[gt.pstart + 1] = make_double2(sp, cp);
      sc[gt.pstart + 2] = make_double2(sl, cl);
      double spl = sp * cl + cp * sl, cpl = cp * cl - sp * sl;
      m.u[0] = make_double2(ct, 0.0);
      m.u[1] = make_double2(-st * cl, -st * sl);
      m.u[2] = make_double2(st * cp, st * sp);
      m.u[3] = make_double2(ct * cpl, ct * spl);
    } else if (gate_param_num(gt.type) == 1) {
      double s, c;
      sincos(th[gt.pstart], &s, &c);
      sc[gt.pstart] = make_double2(s, c);
      m.u[0] = make_double2(c, s);
    }
    gm[g] = m;
  }
}

}  // namespace sqg
