// Batched decomposition: one CTA runs one complete decomposition (BFGS with Powell's
// Z-matrix update, its line search and the restart loop) of one small target, with the
// cost and adjoint gradient evaluated in the CTA's shared memory.  A single launch
// decomposes the whole batch; no host round trip happens per iteration.
//
// Algorithm restated from the reference:
//   src-cpp/common/BFGS_Powell.cpp:70-192 (Optimize), :202-396 (BFGS_iteration),
//   :407-446 (get_search_direction); src-cpp/common/grad_descend.cpp:127-273 (line
//   search), :399-425 (maximal step); restarts: optimization_engines/BFGS.cpp:121-150 and
//   Decomposition_Base.cpp:375-700 (outer loop, tolerance test :742-752).
// The Givens sweep of the Z update is evaluated in parallel from suffix sums of squares
// of Z^T g instead of the sequential hypot chain (same rotations up to rounding).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdlib>
#include <string>

#include "../../include/sqg.h"
#include "gates.cuh"
#include "handle.h"
#include "adam.cuh"
#include "bfgs.cuh"
#include "tile.cuh"

using namespace sqg;


namespace {

constexpr int kDecThreads = 128;
constexpr int kDecVectors = 19;  // P-vectors in shared memory (Sh::x ... Sh::sdv)

struct DecArgs {
  const Gate* gates;
  long long gstride;  // gate records between the lists of consecutive instances (0: one shared list)
  int L, P, n, N, cols, trace_offset, variant;
  const double2* targets;
  long long tstride;
  double* x;
  double* cost;
  int* calls;
  int* iters;
  int B;
  double tol;
  int max_calls, max_outer, loops, early_stop;
  unsigned long long seed;
  double* zglob;        // BFGS matrices in global memory: zslots slots of P * P doubles
  unsigned int* zbits;  // occupancy bitmap of the slots (cleared before the launch)
  int zslots;
  int z_in_smem;
  int cyclic;  // cost and gradient through the environment matrix (dec_eval_cyclic)
  int has_lam;  // 0: the one-chain environment form of a square target, which needs no lambda tiles
  int tgt_in_smem;  // 1: the target is copied to shared memory; 0: read from global memory (L2)
  int chains;  // 2: the two-warp form dec_eval_cyclic2, split at gate `split`
  int split;
  // ADAM engine (k_decompose<kAdam>)
  double eta;
  int adaptive_eta, shift_max;
  double inv_cols;  // 1 / cols (exact for powers of two)
  long long rand_thr;
};

enum { kBfgs = 0, kAdam = 1 };

struct Sh {
  const Gate* gates;    // shared-memory copy of the gate list
  const double2* tgt;  // this instance's target (N x cols, row-major): shared-memory copy or global
  double2 *psi, *lam, *sc;
  GateMat* gm;
  double* R;   // [L][8] reduced 2x2 overlaps of the reverse sweep
  int* pgate;  // gate owning each parameter
  int* pg;     // indices of the parametric gates
  int npg;
  double *x, *g, *d, *x0, *g0, *gbest, *ztg, *delta, *gamma, *gtz, *nz, *bestx, *guess, *S, *cs, *zs, *v, *vp, *sdv;
  double *Z, *redd, *tot, *scratch;
};

// Gate matrices of parameter vector xv: one sincos per parameter (threads over
// parameters, so every warp instruction of the FP64 series works on full warps), then the
// 2x2 kernels from the stored (sin, cos) (threads over gates).  Same formulas as
// build_gate_mats.
__device__ void dec_build(const DecArgs& a, const Sh& sh, const double* xv) {
  for (int p = threadIdx.x; p < a.P; p += blockDim.x) {
    double s, c;
    sincos(xv[p], &s, &c);
    sh.sc[p] = make_double2(s, c);
  }
  __syncthreads();
  for (int g = threadIdx.x; g < a.L; g += blockDim.x) {
    const Gate gt = sh.gates[g];
    GateMat m;
    m.u[0] = m.u[1] = m.u[2] = m.u[3] = make_double2(0.0, 0.0);
    if (gt.type == G_U3) {
      const double st = sh.sc[gt.pstart].x, ct = sh.sc[gt.pstart].y;
      const double sp = sh.sc[gt.pstart + 1].x, cp = sh.sc[gt.pstart + 1].y;
      const double sl = sh.sc[gt.pstart + 2].x, cl = sh.sc[gt.pstart + 2].y;
      const double spl = sp * cl + cp * sl, cpl = cp * cl - sp * sl;
      m.u[0] = make_double2(ct, 0.0);
      m.u[1] = make_double2(-st * cl, -st * sl);
      m.u[2] = make_double2(st * cp, st * sp);
      m.u[3] = make_double2(ct * cpl, ct * spl);
    } else if (gate_param_num(gt.type) == 1) {
      m.u[0] = make_double2(sh.sc[gt.pstart].y, sh.sc[gt.pstart].x);
    }
    sh.gm[g] = m;
  }
}

// Cost of the variant from the trace tr and gradient from the buffered overlaps
// sh.R (src-cpp/decomposition/Optimization_Interface.cpp:1395-1430 for the gradient
// components, FROBENIUS_NORM with the reference's (1 - t/N) - 1 rounding).
__device__ double dec_finish(const DecArgs& a, const Sh& sh, double2 tr, double* gv) {
  const double* Rb = sh.R;
  double f;
  const double dc = a.cols, inv_dc = a.inv_cols;
  // x / cols and x * (1 / cols) round identically when cols is a power of two
  const bool pow2 = (a.cols & (a.cols - 1)) == 0;
  double cx = 0.0, cy = 0.0;  // HILBERT_SCHMIDT_TEST / INFIDELITY: grad = cx t.x - cy t.y
  if (a.variant == SQG_FROBENIUS_NORM) {
    f = 1.0 - (pow2 ? tr.x * inv_dc : tr.x / dc);
  } else if (a.variant == SQG_HILBERT_SCHMIDT_TEST) {
    double d = 1.0 / dc;
    f = 1.0 - d * d * (tr.x * tr.x + tr.y * tr.y);
    cx = -2.0 * d * d * tr.x;
    cy = 2.0 * d * d * tr.y;
  } else {
    f = 1.0 - ((tr.x * tr.x + tr.y * tr.y) / dc + 1) / (dc + 1);
    cx = -2.0 / dc / (dc + 1) * tr.x;
    cy = 2.0 / dc / (dc + 1) * tr.y;
  }
  auto grad = [&](double tx, double ty) {
    if (a.variant == SQG_FROBENIUS_NORM) return (1.0 - (pow2 ? tx * inv_dc : tx / dc)) - 1.0;
    return cx * tx - cy * ty;
  };
  // one thread per parametric gate: the three U3 derivatives share their products and
  // their kernels' zero entries (deriv_kernel) are skipped; the contractions keep the
  // order of contract_derivative
  for (int j = threadIdx.x; j < sh.npg; j += blockDim.x) {
    const int g = sh.pg[j];
    const Gate gt = sh.gates[g];
    const double* R = Rb + g * 8;
    if (gt.type == G_U3) {
      const double2* s3 = sh.sc + gt.pstart;
      const double st = s3[0].x, ct = s3[0].y, sp = s3[1].x, cp = s3[1].y, sl = s3[2].x, cl = s3[2].y;
      const double spl = sp * cl + cp * sl, cpl = cp * cl - sp * sl;
      const double r0 = R[0], i0 = R[1], r1 = R[2], i1 = R[3], r2 = R[4], i2 = R[5], r3 = R[6], i3 = R[7];
      // theta: (-st, 0), (-ct cl, -ct sl), (ct cp, ct sp), (-st cpl, -st spl)
      double tx = -st * r0, ty = -st * i0;
      double dx = -ct * cl, dy = -ct * sl;
      tx = fma(dx, r1, fma(-dy, i1, tx));
      ty = fma(dx, i1, fma(dy, r1, ty));
      dx = ct * cp;
      dy = ct * sp;
      tx = fma(dx, r2, fma(-dy, i2, tx));
      ty = fma(dx, i2, fma(dy, r2, ty));
      dx = -st * cpl;
      dy = -st * spl;
      tx = fma(dx, r3, fma(-dy, i3, tx));
      ty = fma(dx, i3, fma(dy, r3, ty));
      gv[gt.pstart] = grad(tx, ty);
      // phi: 0, 0, (-st sp, st cp), (-ct spl, ct cpl)
      const double ex = -ct * spl, ey = ct * cpl;
      dx = -st * sp;
      dy = st * cp;
      tx = fma(dx, r2, -dy * i2);
      ty = fma(dx, i2, dy * r2);
      tx = fma(ex, r3, fma(-ey, i3, tx));
      ty = fma(ex, i3, fma(ey, r3, ty));
      gv[gt.pstart + 1] = grad(tx, ty);
      // lambda: 0, (st sl, -st cl), 0, (-ct spl, ct cpl)
      dx = st * sl;
      dy = -st * cl;
      tx = fma(dx, r1, -dy * i1);
      ty = fma(dx, i1, dy * r1);
      tx = fma(ex, r3, fma(-ey, i3, tx));
      ty = fma(ex, i3, fma(ey, r3, ty));
      gv[gt.pstart + 2] = grad(tx, ty);
    } else {
      for (int k = 0; k < gate_param_num(gt.type); k++) {
        const double2 t = contract_derivative(gt, sh.sc, k, R);
        gv[gt.pstart + k] = grad(t.x, t.y);
      }
    }
  }
  __syncthreads();
  return f;
}

// Barrier among the first aw warps of the CTA (the ones that run the sweep).
__device__ __forceinline__ void sweep_sync(int aw) {
  if (aw == (int)(blockDim.x >> 5))
    __syncthreads();
  else if (aw == 1)
    __syncwarp();
  else
    asm volatile("bar.sync 1, %0;" ::"r"(aw * 32) : "memory");
}

// Overlap of gate gt from the environment matrix m (N x N, m[c * N + r] = M[r][c]):
// R_ab = sum over the other qubits of M[(b, rest)][(a, rest)] (for a controlled gate only
// the rest with the control bit set), written as R[2 * (2a + b) + {0, 1}].  Warp 0 only.
__device__ __forceinline__ void cyclic_overlap(const double2* m, int n, int N, const Gate& gt, double* R) {
  const int lane = threadIdx.x & 31;
  const bool ctrl = gate_controlled(gt.type);
  const int entries = 4 << (ctrl ? n - 2 : n - 1);
  double2 v = make_double2(0.0, 0.0);
  for (int j = lane; j < entries; j += 32) {
    const int q = j & 3, ri = j >> 2;
    const int rest = ctrl ? pair_index2(ri, gt.target, gt.control) : pair_index1(ri, gt.target);
    const int row = rest | ((q & 1) << gt.target), col = rest | ((q >> 1) << gt.target);
    const double2 e = m[col * N + row];
    if (j == lane) {
      v = e;
    } else {
      v.x += e.x;
      v.y += e.y;
    }
  }
  const int span = entries < 32 ? entries : 32;
  for (int o = 4; o < span; o <<= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  if (lane < 4) {
    R[2 * lane] = v.x;
    R[2 * lane + 1] = v.y;
  }
}

// Cost and adjoint gradient in the cyclic form, for targets with cols >= 3N/4 columns.
// With psi_{k-1} = G_{k-1} ... G_0 T (the state in front of gate k) and lambda_k =
// G_{k+1}^dagger ... G_{L-1}^dagger E (E: the columns e_{j + trace_offset}), the overlap
// R_ab = sum conj(lambda_a) psi_b of gate k is a partial trace of the N x N matrix
// M_k = psi_{k-1} lambda_k^dagger.  M_0 = T E^dagger G_{L-1} ... G_1 and
// M_{k+1} = G_k M_k G_{k+1}^dagger, so one matrix carried through the circuit replaces the
// state and adjoint sweeps and their per-gate inner products; tr(G_0 M_0) =
// tr(E^dagger U T) is the trace of the cost.  M is a 2n-qubit register (row bits low,
// column bits high): multiplying by G from the left applies G to qubit t, from the right
// applies G^T (G^dagger: conj G) to qubit t + n.
__device__ double dec_eval_cyclic(const DecArgs& a, const Sh& sh, const double* xv, double* gv, int b) {
  const int n = a.n, N = a.N, NN = N * N, cols = a.cols, off = a.trace_offset, L = a.L;
  dec_build(a, sh, xv);
  double2* m = sh.psi;  // N * N entries: psi alone when cols = N, else psi and the contiguous lam
  const double2* T = sh.tgt;
  // M_0[r][j + off] = T[r][j] (m column-major), zero outside the target's columns; walked in
  // the target's row-major order so that a target read from L2 is read coalesced
  if (cols != N || off != 0)
    for (int e = threadIdx.x; e < NN; e += blockDim.x) {
      const int j = (e >> n) - off;
      if (j < 0 || j >= cols) m[e] = make_double2(0.0, 0.0);
    }
  for (int e = threadIdx.x; e < N * cols; e += blockDim.x) {
    const int r = e / cols, j = e - r * cols;
    m[(j + off) * N + r] = T[e];
  }
  __syncthreads();
  const int aw = min((int)(blockDim.x >> 5), (NN / 2 + 31) >> 5);
  if ((int)(threadIdx.x >> 5) < aw) {
    auto right = [&](int g, int orient) {
      Gate gs = sh.gates[g];
      gs.target += n;
      if (gate_controlled(gs.type)) gs.control += n;
      tile_apply(m, NN, 2 * n, 1, gs, make_op(gs.type, sh.gm[g], orient));
      sweep_sync(aw);
    };
#pragma unroll 1
    for (int g = L - 1; g >= 1; g--) right(g, ORIENT_TRANS);
    // for g = 0 .. L-1: [overlap of G_g] [M <- G_g M, except g = L-1 > 0] [trace at g = 0]
    // [M <- M G_{g+1}^dagger, g < L-1], as a loop of four sub-steps per gate with one
    // gate-application site (a small code footprint, as in dec_eval_cyclic2)
#pragma unroll 1
    for (int s = 0; s < 4 * L; s++) {
      const int g = s >> 2, sub = s & 3;
      const Gate gt = sh.gates[g];
      int act = 0, gk = g, orient = ORIENT_FWD;  // act: 1 apply, 2 overlap, 3 trace
      bool shift = false;
      if (sub == 0 && gate_param_num(gt.type) > 0) act = 2;
      else if (sub == 1 && (g == 0 || g < L - 1)) act = 1;
      else if (sub == 2 && g == 0) act = 3;
      else if (sub == 3 && g < L - 1) { act = 1; shift = true; gk = g + 1; orient = ORIENT_CONJ; }
      if (act == 1) {
        Gate x = sh.gates[gk];
        if (shift) {
          x.target += n;
          if (gate_controlled(x.type)) x.control += n;
        }
        tile_apply(m, NN, 2 * n, 1, x, make_op(x.type, sh.gm[gk], orient));
        sweep_sync(aw);
      } else if (act == 2) {
        if (threadIdx.x < 32) cyclic_overlap(m, n, N, gt, sh.R + g * 8);
        sweep_sync(aw);
      } else if (act == 3) {
        if (threadIdx.x < 32) {
          const int lane = threadIdx.x;
          double2 v = lane < N ? m[lane * N + lane] : make_double2(0.0, 0.0);
          for (int i = lane + 32; i < N; i += 32) {  // N = 64: two diagonal entries per lane
            v.x += m[i * N + i].x;
            v.y += m[i * N + i].y;
          }
          for (int o = 1; o < min(N, 32); o <<= 1) {  // lanes 0..min(N, 32)-1 end with the full sum
            v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
            v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
          }
          if (lane == 0) {
            sh.redd[0] = v.x;
            sh.redd[1] = v.y;
          }
        }
        sweep_sync(aw);
      }
    }
  }
  __syncthreads();
  const double2 tr = make_double2(sh.redd[0], sh.redd[1]);
  return dec_finish(a, sh, tr, gv);
}

// Two-warp form of dec_eval_cyclic for square targets (cols = N, no trace offset) with
// N^2 / 2 <= 32 amplitude pairs, so that one warp holds one environment matrix.  Warp 0
// builds psi_{h-1} = G_{h-1} ... G_0 T and warp 1 W = lambda_h^dagger = G_{L-1} ... G_{h+1}
// (right products on the identity) at the same time; M_h = psi_{h-1} W is one N x N
// product shared by both warps; then warp 1 runs M_{k+1} = G_k M_k G_{k+1}^dagger up to
// gate L-1 (taking tr(G_h M_h) on the way) and warp 0 runs M_k = G_k^dagger M_{k+1}
// G_{k+1} down to gate 0, each taking the overlaps of its own gates.  The FP64 work is that
// of the one-warp form plus the product; the latency of an evaluation is about halved,
// which is what a CTA running alone (the end of a batch, small batches) waits for.
__device__ double dec_eval_cyclic2(const DecArgs& a, const Sh& sh, const double* xv, double* gv) {
  const int n = a.n, N = a.N, NN = N * N, L = a.L, h = a.split;
  dec_build(a, sh, xv);
  __syncthreads();
  double2* mA = sh.psi;
  double2* mB = sh.lam;  // cols = N: each region holds N * N entries
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  auto shifted = [&](int g) {
    Gate gs = sh.gates[g];
    gs.target += n;
    if (gate_controlled(gs.type)) gs.control += n;
    return gs;
  };
  // Each phase of each chain is one loop with one gate-application site (the gate, the side
  // and the orientation are chosen per step), so the evaluation's code stays small: the eight
  // CTAs of an SM run it and the BFGS update in different phases out of one instruction cache.
  double2* const m = warp == 0 ? mA : mB;
  if (warp < 2) {
    for (int e = lane; e < NN; e += 32)
      m[e] = warp == 0 ? sh.tgt[(e & (N - 1)) * N + (e >> n)]
                       : make_double2((e & (N - 1)) == (e >> n) ? 1.0 : 0.0, 0.0);
    __syncwarp();
    // warp 0: psi_{h-1} = G_{h-1} ... G_0 T; warp 1: W = G_{L-1} ... G_{h+1} from the right
    const int steps = warp == 0 ? h : L - 1 - h;
#pragma unroll 1
    for (int s = 0; s < steps; s++) {
      const int k = warp == 0 ? s : L - 1 - s;
      const Gate gt = warp == 0 ? sh.gates[k] : shifted(k);
      tile_apply_by(m, NN, 2 * n, 1, gt, make_op(gt.type, sh.gm[k], warp == 0 ? ORIENT_FWD : ORIENT_TRANS), lane,
                    32);
      __syncwarp();
    }
  }
  if (warp < 2) {
    // M_h[y][x] = sum_c psi[y][c] W[c][x], entry x * N + y, one per thread of the two warps
    asm volatile("bar.sync 2, 64;" ::: "memory");
    const int e = threadIdx.x;
    double2 acc = make_double2(0.0, 0.0);
    if (e < NN) {
      const int x = e >> n, y = e & (N - 1);
      for (int c = 0; c < N; c++) {
        const double2 p = mA[c * N + y], w = mB[x * N + c];
        acc.x = fma(p.x, w.x, fma(-p.y, w.y, acc.x));
        acc.y = fma(p.x, w.y, fma(p.y, w.x, acc.y));
      }
    }
    asm volatile("bar.sync 2, 64;" ::: "memory");
    if (e < NN) {
      mA[e] = acc;
      mB[e] = acc;
    }
    asm volatile("bar.sync 2, 64;" ::: "memory");
  }
  if (warp < 2) {
    // warp 1, for k = h .. L-1: [overlap of G_k] [M <- G_k M, except k = L-1 > h] [trace at
    // k = h] [M <- M G_{k+1}^dagger, k < L-1];  warp 0, for k = h-1 .. 0: [M <- G_k^dagger M]
    // [M <- M G_{k+1}] [overlap of G_k].  Four sub-steps per gate, in that order.
    const int gates = warp == 0 ? h : L - h;
#pragma unroll 1
    for (int s = 0; s < 4 * gates; s++) {
      const int k = warp == 0 ? h - 1 - (s >> 2) : h + (s >> 2), sub = s & 3;
      const bool param = gate_param_num(sh.gates[k].type) > 0;
      int act = 0, gk = k, orient = ORIENT_FWD;  // act: 1 apply, 2 apply shifted, 3 overlap, 4 trace
      bool right = false;
      if (warp == 1) {
        if (sub == 0 && param) act = 3;
        else if (sub == 1 && (k == h || k < L - 1)) act = 1;
        else if (sub == 2 && k == h) act = 4;
        else if (sub == 3 && k < L - 1) { act = 1; right = true; gk = k + 1; orient = ORIENT_CONJ; }
      } else {
        if (sub == 0) { act = 1; orient = ORIENT_ADJ; }
        else if (sub == 1) { act = 1; right = true; gk = k + 1; orient = ORIENT_TRANS; }
        else if (sub == 2 && param) act = 3;
      }
      if (act == 1) {
        const Gate gt = right ? shifted(gk) : sh.gates[gk];
        tile_apply_by(m, NN, 2 * n, 1, gt, make_op(gt.type, sh.gm[gk], orient), lane, 32);
        __syncwarp();
      } else if (act == 3) {
        cyclic_overlap(m, n, N, sh.gates[k], sh.R + k * 8);
        __syncwarp();
      } else if (act == 4) {  // tr(G_h M_h) = tr(E^dagger U T)
        double2 v = lane < N ? m[lane * N + lane] : make_double2(0.0, 0.0);
        for (int o = 1; o < N; o <<= 1) {
          v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
          v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        }
        if (lane == 0) {
          sh.redd[0] = v.x;
          sh.redd[1] = v.y;
        }
        __syncwarp();
      }
    }
  }
  __syncthreads();
  return dec_finish(a, sh, make_double2(sh.redd[0], sh.redd[1]), gv);
}

// Cost and gradient of parameter vector xv (smem) for instance b; gradient into gv.  FORM
// (a template parameter, so that each kernel carries the code of one form only):
// kFormSweep state sweeps, kFormCyclic environment matrix on all warps, kFormTwoChains the
// two-warp environment matrix.  Not inlined: the BFGS driver calls it from two places (first
// evaluation, line search), and one shared copy of its code keeps the instruction cache warm
// for the eight CTAs of an SM, which run it and the BFGS update in different phases (measured
// on GB300: +5.8% decompositions/s, identical evaluation counts, although more registers spill
// across the call).
enum { kFormSweep = 0, kFormCyclic = 1, kFormTwoChains = 2 };

template <int FORM>
__device__ __noinline__ double dec_eval(const DecArgs& a, const Sh& sh, const double* xv, double* gv, int b) {
  if constexpr (FORM == kFormTwoChains) return dec_eval_cyclic2(a, sh, xv, gv);
  if constexpr (FORM == kFormCyclic) return dec_eval_cyclic(a, sh, xv, gv, b);
  const int N = a.N, cols = a.cols, off = a.trace_offset;
  dec_build(a, sh, xv);
  const double2* T = sh.tgt;
  for (int e = threadIdx.x; e < N * cols; e += blockDim.x) {
    int r = e / cols, c = e - r * cols;
    sh.psi[c * N + r] = T[e];
    sh.lam[c * N + r] = make_double2(r == c + off ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
  for (int g = 0; g < a.L; g++) {
    Gate gt = sh.gates[g];
    tile_apply(sh.psi, N, a.n, cols, gt, make_op(gt.type, sh.gm[g], ORIENT_FWD));
    __syncthreads();
  }
  double2 tr = tile_trace(sh.psi, N, cols, 0, off, sh.scratch);
  double* Rb = sh.R;
  // buffer each gate's overlap; the derivative contractions run afterwards for all
  // parameters at once on full warps
  adjoint_sweep(sh.psi, sh.lam, N, a.n, cols, sh.gates, sh.gm, sh.sc, a.L, sh.redd, sh.tot,
                [&](int g, const Gate&, const double* R) {
                  if (threadIdx.x < 8) Rb[g * 8 + threadIdx.x] = R[threadIdx.x];
                },
                [](int) {});
  __syncthreads();
  return dec_finish(a, sh, tr, gv);
}


// BFGS_Powell::Optimize from sh.x (updated in place).  Returns the final cost.  The
// evaluation budget a.max_calls applies to this run (a new BFGS_Powell with its own call
// count per restart, optimization_engines/BFGS.cpp:121-125); calls and iters accumulate
// over the runs of the decomposition.
template <int FORM, class ZA>
__device__ double dec_bfgs(const DecArgs& a, const Sh& sh, int b, int& calls, int& iters, const ZA& za) {
  int run = 0;
  const int P = a.P;
  double* Z = sh.Z;
  const BfgsVecs bv = {sh.Z, sh.x, sh.x0, sh.g, sh.g0, sh.gbest, sh.d, sh.delta, sh.gamma, sh.v, sh.vp, sh.cs,
                       sh.ztg, sh.zs, sh.S, sh.sdv, sh.nz, sh.gtz, sh.redd, sh.scratch};
  for (int i = threadIdx.x; i < P * P; i += blockDim.x) za.st(Z + i, (i % (P + 1)) == 0 ? 1.0 : 0.0);
  double norm_Z = -1.0;
  double f = dec_eval<FORM>(a, sh, sh.x, sh.g, b);
  calls++;
  run++;
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    sh.cs[i] = 1.0;
    sh.ztg[i] = sh.g[i];
    sh.zs[i] = sh.g[i];
  }
  __syncthreads();
  if (a.early_stop && f < a.tol) return f;
  double fprev = fabs(f + f + 1.0);
  for (;;) {
    double dg, max_step, gn;
    bfgs_direction(P, bv, dg, max_step, gn, za);
    if (gn <= 1e-19 * 1e-19 || dg >= 0.0 || f >= fprev) break;
    fprev = f;
    if (run >= a.max_calls) break;
    iters++;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
      sh.x0[i] = sh.x[i];
      sh.g0[i] = sh.g[i];
      sh.gbest[i] = sh.g[i];
    }
    __syncthreads();
    double step = fmin(1.0, max_step);
    double f_low = f, f_high = f, s_high = max_step, s_low = 0.0, s_best = 0.0, f_best = f, dg_best = fabs(dg);
    double dg_high = 0.0;
    for (int it = 0; it < 50; it++) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) sh.x[i] = sh.x0[i] + step * sh.d[i];
      __syncthreads();
      f = dec_eval<FORM>(a, sh, sh.x, sh.g, b);
      calls++;
      run++;
      if (a.early_stop && f < a.tol) return f;
      double dgc = dot(sh.d, sh.g, P, sh.scratch);
      if (f < f_best || fabs(dgc) < dg_best) {
        s_best = step;
        f_best = f;
        dg_best = fabs(dgc);
        for (int i = threadIdx.x; i < P; i += blockDim.x) sh.gbest[i] = sh.g[i];
        __syncthreads();
      }
      if (run == a.max_calls) break;
      if (f < f_low + step * 0.1 * dg) {
        if (dgc >= dg * 0.7) break;
        s_low = step;
        f_low = f;
      } else {
        s_high = step;
        f_high = f;
        dg_high = dgc;
      }
      if (it == 0 || s_low > 0.0) {
        double dlf = (f_high - f_low) / (s_high - s_low) * 2.0 - dg_high;
        double scale = -dlf * 0.5 / (dg_high - dlf);
        scale = fmax(0.1, scale);
        step = s_low + scale * (s_high - s_low);
      } else {
        step = step * 0.1;
        if (step < kNumPrecision) break;
      }
    }
    if (step != s_best) {
      step = s_best;
      f = f_best;
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        sh.g[i] = sh.gbest[i];
        sh.x[i] = sh.x0[i] + step * sh.d[i];
      }
      __syncthreads();
    }
    if (step == 0.0) break;
    norm_Z = bfgs_update(P, bv, norm_Z, za);
  }
  return f;
}

// SQUANDER's ADAM engine for one target (adam.cuh) with the evaluation of this kernel:
// starts from sh.x, leaves the best point in sh.bestx and returns the minimum.  f0_vec and
// dec_vec are the engine's 100- and 20-entry windows.
template <int FORM>
__device__ double dec_adam(const DecArgs& a, const Sh& sh, int b, int& calls, int& shifts, double cur_min,
                           unsigned long long& rng, double* f0_vec, int* dec_vec) {
  const AdamConfig cfg = {a.P, a.tol, a.eta, a.adaptive_eta, a.shift_max, a.rand_thr};
  const AdamVecs v = {sh.x, sh.g, sh.bestx, sh.v, sh.vp, sh.S, sh.sdv, f0_vec, dec_vec, sh.redd};
  adam_powers(v, a.P);
  AdamRun s;
  adam_begin(s, cfg, v, cur_min);
  for (int it = 0; it < a.max_calls; it++) {
    const double f0 = dec_eval<FORM>(a, sh, sh.x, sh.g, b);
    calls++;
    if (adam_after_eval(s, cfg, v, f0, rng)) break;
  }
  shifts += s.shift_cnt;
  return s.cur_min;
}

// Shared-memory layout common to the decomposition and evaluation kernels (dec_smem_bytes
// without the optimizer's own part): gate list, target of instance b, state matrices, gate
// matrices, per-gate overlaps, parameter maps, kDecVectors P-vectors and reduction scratch.
// Loads the gate list and the target; returns the first free byte.  The caller
// synchronises before use.
__device__ char* dec_setup(const DecArgs& a, Sh& sh, int b, char* p) {
  const int P = a.P, L = a.L, NC = a.N * a.cols;
  auto take = [&](size_t bytes) { char* r = p; p += (bytes + 15) / 16 * 16; return r; };
  Gate* gsh = (Gate*)take(sizeof(Gate) * max(L, 1));
  sh.gates = gsh;
  double2* tsh = a.tgt_in_smem ? (double2*)take(sizeof(double2) * NC) : nullptr;
  sh.tgt = a.tgt_in_smem ? tsh : a.targets + (long long)b * a.tstride;
  sh.psi = (double2*)take(sizeof(double2) * NC);
  sh.lam = a.has_lam ? (double2*)take(sizeof(double2) * NC) : nullptr;
  sh.gm = (GateMat*)take(sizeof(GateMat) * max(L, 1));
  sh.sc = (double2*)take(sizeof(double2) * max(P, 1));
  sh.R = (double*)take(sizeof(double) * 8 * max(L, 1));
  sh.pgate = (int*)take(sizeof(int) * max(P, 1));
  sh.pg = (int*)take(sizeof(int) * max(L, 1));
  sh.npg = 0;
  const Gate* gl = a.gates + (long long)b * a.gstride;  // this instance's gate list
  for (int g = 0; g < L; g++)
    if (gate_param_num(gl[g].type) > 0) {
      if (threadIdx.x == 0) sh.pg[sh.npg] = g;
      sh.npg++;
    }
  double** vecs[] = {&sh.x, &sh.g, &sh.d, &sh.x0, &sh.g0, &sh.gbest, &sh.ztg, &sh.delta, &sh.gamma,
                     &sh.gtz, &sh.nz, &sh.bestx, &sh.guess, &sh.S, &sh.cs, &sh.zs, &sh.v, &sh.vp, &sh.sdv};
  static_assert(sizeof(vecs) / sizeof(vecs[0]) == kDecVectors, "dec_smem_bytes counts kDecVectors vectors");
  for (double** v : vecs) *v = (double*)take(sizeof(double) * max(P, 1));
  sh.redd = (double*)take(sizeof(double) * kTileMaxWarps * 8);
  sh.tot = (double*)take(sizeof(double) * 8);
  sh.scratch = (double*)take(sizeof(double) * kTileMaxWarps);
  sh.Z = nullptr;
  if (a.tgt_in_smem)
    for (int e = threadIdx.x; e < NC; e += blockDim.x) tsh[e] = a.targets[(long long)b * a.tstride + e];
  for (int g = threadIdx.x; g < L; g += blockDim.x) {
    const Gate gt = gl[g];
    gsh[g] = gt;
    for (int k = 0; k < gate_param_num(gt.type); k++) sh.pgate[gt.pstart + k] = g;
  }
  return p;
}

// BFGS matrices in global memory are indexed by a slot that a CTA holds while it runs, not by
// its target: there are only as many slots as CTAs of the launch can be resident at once, so
// the matrices of a 4096-target launch stay within L2 instead of spreading over 4096 x 69 KB
// and being written back to HBM.  A CTA claims the lowest free slot it finds (one atomicOr per
// attempt on the occupancy bitmap) and clears its bit when it finishes; the bitmap is never
// full when a CTA starts because fewer CTAs than slots are then resident.  Each scan is
// bounded; after kClaimScans scans without a free slot the CTA gives up (-1).
constexpr int kClaimScans = 1024;

__device__ int claim_z_slot(unsigned int* bits, int slots) {
  const int words = (slots + 31) / 32;
  for (int scan = 0; scan < kClaimScans; ++scan) {
    for (int w = 0; w < words; ++w) {
      const unsigned int valid = (w == words - 1 && (slots & 31)) ? ((1u << (slots & 31)) - 1u) : 0xffffffffu;
      unsigned int seen = *((volatile unsigned int*)&bits[w]);
      // each pass either takes a bit or marks one more bit as taken: at most 32 passes
      for (int pass = 0; pass < 32; ++pass) {
        const unsigned int free_bits = ~seen & valid;
        if (!free_bits) break;
        const int bit = __ffs(free_bits) - 1;
        const unsigned int old = atomicOr(&bits[w], 1u << bit);
        if (!(old & (1u << bit))) {
          __threadfence();
          return w * 32 + bit;
        }
        seen = old | (1u << bit);
      }
    }
  }
  return -1;
}

__device__ void release_z_slot(unsigned int* bits, int slot) {
  __threadfence();  // this CTA's writes to the slot are ordered before its release
  atomicAnd(&bits[slot >> 5], ~(1u << (slot & 31)));
}

// Batched cost and gradient through the environment-matrix evaluation, one CTA per
// parameter vector b (theta row b, target b * a.tstride; tstride 0 shares one target).
template <int FORM>
__global__ void __launch_bounds__(kDecThreads, 6) k_env_costgrad(DecArgs a, const double* __restrict__ theta,
                                                                 double* __restrict__ cost, double* __restrict__ grad) {
  extern __shared__ double2 smem2[];
  const int b = blockIdx.x;
  if (b >= a.B) return;
  Sh sh;
  dec_setup(a, sh, b, reinterpret_cast<char*>(smem2));
  for (int i = threadIdx.x; i < a.P; i += blockDim.x) sh.x[i] = theta[(long long)b * a.P + i];
  __syncthreads();
  const double f = dec_eval<FORM>(a, sh, sh.x, sh.g, b);
  for (int i = threadIdx.x; i < a.P; i += blockDim.x) grad[(long long)b * a.P + i] = sh.g[i];
  if (threadIdx.x == 0) cost[b] = f;
}

// At most 80 registers (6 CTAs of 128 threads per SM): the evaluation keeps only one warp
// per CTA busy at n = 3, so resident CTAs are what hides FP64 and shared-memory latency
// (measured 7470 vs 7103 decompositions/s with the unconstrained 126 registers).  ZG: the
// BFGS matrices live in global slots and are accessed with the L2 evict_last policy
// (ZKeepL2); otherwise they are in shared memory (or absent, for ADAM).
template <int OPT, int FORM, bool ZG>
__global__ void __launch_bounds__(kDecThreads, 6) k_decompose(DecArgs a) {
  extern __shared__ double2 smem2[];
  const int b = blockIdx.x;
  if (b >= a.B) return;
  const int P = a.P;
  Sh sh;
  char* p = dec_setup(a, sh, b, reinterpret_cast<char*>(smem2));
  auto take = [&](size_t bytes) { char* r = p; p += (bytes + 15) / 16 * 16; return r; };
  double* f0_vec = nullptr;
  int* dec_vec = nullptr;
  if (OPT == kAdam) {
    f0_vec = (double*)take(sizeof(double) * 100);
    dec_vec = (int*)take(sizeof(int) * 20);
    sh.Z = nullptr;
  } else if (a.z_in_smem) {
    if constexpr (ZG) {  // the L2-kept accessors need Z in global memory: not this launch
      if (threadIdx.x == 0) {
        a.cost[b] = __longlong_as_double(0x7ff8000000000000LL);
        a.calls[b] = -1;
        if (a.iters) a.iters[b] = -1;
      }
      return;
    }
    sh.Z = (double*)take(sizeof(double) * P * P);
  } else {
    __shared__ int z_slot;
    if (threadIdx.x == 0) z_slot = claim_z_slot(a.zbits, a.zslots);
    __syncthreads();
    if (z_slot < 0) {  // no slot (not expected): report the instance as failed
      if (threadIdx.x == 0) {
        a.cost[b] = __longlong_as_double(0x7ff8000000000000LL);
        a.calls[b] = -1;
        if (a.iters) a.iters[b] = -1;
      }
      return;
    }
    sh.Z = a.zglob + (long long)z_slot * P * P;
  }

  for (int i = threadIdx.x; i < P; i += blockDim.x) sh.guess[i] = a.x[(long long)b * P + i];
  __syncthreads();
  double best = INFINITY;
  int calls = 0, iters = 0;
  if (OPT == kAdam) {
    // one engine call per outer iteration from the best point so far, the running minimum
    // carried over (Decomposition_Base keeps current_minimum across them)
    unsigned long long rng = a.seed + (unsigned long long)b * 7919ULL;
    double cur_min = DBL_MAX;
    for (int outer = 0; outer < a.max_outer; outer++) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) sh.x[i] = sh.guess[i];
      __syncthreads();
      cur_min = dec_adam<FORM>(a, sh, b, calls, iters, cur_min, rng, f0_vec, dec_vec);
      for (int i = threadIdx.x; i < P; i += blockDim.x) sh.guess[i] = sh.bestx[i];
      __syncthreads();
      if (fabs(cur_min) < a.tol) break;
    }
    best = cur_min;
  }
  unsigned long long ctr = a.seed * 0x2545F4914F6CDD1DULL + (unsigned long long)b * 0x9E3779B97F4A7C15ULL;
  bool done = OPT == kAdam;
  for (int outer = 0; outer < a.max_outer && !done; outer++) {
    for (int loop = 0; loop < a.loops; loop++) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) sh.x[i] = sh.guess[i];
      __syncthreads();
      double f;
      if constexpr (ZG)
        f = dec_bfgs<FORM>(a, sh, b, calls, iters, ZKeepL2());
      else
        f = dec_bfgs<FORM>(a, sh, b, calls, iters, ZMem{});
      for (int i = threadIdx.x; i < P; i += blockDim.x) sh.guess[i] = sh.x[i];
      __syncthreads();
      if (f < best) {
        best = f;
        for (int i = threadIdx.x; i < P; i += blockDim.x) {
          sh.bestx[i] = sh.x[i];
          sh.guess[i] = sh.x[i] + u01(ctr + i) * kTwoPi / 100.0;
        }
        ctr += 0x100000001ULL * (unsigned long long)(P + 1);
        __syncthreads();
      }
      if (a.early_stop && best < a.tol) {
        done = true;
        break;
      }
    }
    for (int i = threadIdx.x; i < P; i += blockDim.x) sh.guess[i] = sh.bestx[i];
    __syncthreads();
    if (fabs(best) < a.tol) done = true;
  }
  for (int i = threadIdx.x; i < P; i += blockDim.x) a.x[(long long)b * P + i] = sh.bestx[i];
  if (threadIdx.x == 0) {
    a.cost[b] = best;
    a.calls[b] = calls;
    if (a.iters) a.iters[b] = iters;
  }
  if (OPT == kBfgs && !a.z_in_smem) {
    __syncthreads();  // every thread is done with Z
    if (threadIdx.x == 0) release_z_slot(a.zbits, (int)((sh.Z - a.zglob) / ((long long)P * P)));
  }
}

bool use_cyclic(const sqg_circuit* c, int cols);
bool use_two_chains();

// The lambda tiles are needed by every evaluation form except the one-chain environment form
// of a square target, whose environment matrix (N * N entries) fits in the psi tiles.
bool dec_needs_lam(const sqg_circuit* c, int cols) {
  if (!use_cyclic(c, cols) || cols != c->N) return true;
  return c->N * c->N / 2 <= 32 && c->L >= 2 && use_two_chains();
}

// Threads of a decomposition CTA: one per parameter for the vector and Z-matrix work, at least
// two warps; four at six qubits, where shared memory admits few CTAs per SM and the
// evaluation's 2048 amplitude pairs per gate keep every warp busy.
int dec_threads(const sqg_circuit* c) {
  if (c->n >= 6) return kDecThreads;
  return std::min(kDecThreads, std::max(64, (c->P + 31) / 32 * 32));
}

// Shared memory of one decomposition CTA with the target (tgt) and the BFGS matrix Z (z) on
// chip or not; adam: the ADAM engine's extra windows instead of Z.
size_t dec_smem_layout(const sqg_circuit* c, int cols, bool tgt, bool z, bool adam) {
  auto r16 = [](size_t v) { return (v + 15) / 16 * 16; };
  size_t P = std::max(c->P, 1), L = std::max(c->L, 1), NC = (size_t)c->N * cols;
  // psi, lambda unless the form needs none, the target unless it stays in global memory
  const size_t tiles = 1 + (dec_needs_lam(c, cols) ? 1 : 0) + (tgt ? 1 : 0);
  size_t s = r16(sizeof(Gate) * L) + tiles * r16(sizeof(double2) * NC) + r16(sizeof(GateMat) * L) + r16(sizeof(double2) * P) +
             r16(sizeof(double) * 8 * L) + r16(sizeof(int) * P) + r16(sizeof(int) * L) +
             kDecVectors * r16(sizeof(double) * P) + r16(sizeof(double) * kTileMaxWarps * 8) + r16(sizeof(double) * 8) +
             r16(sizeof(double) * kTileMaxWarps);
  if (adam) return s + r16(sizeof(double) * 100) + r16(sizeof(int) * 20);
  if (z) s += r16(sizeof(double) * P * P);
  return s;
}

// Decomposition CTAs one SM holds with `threads` threads and `smem` bytes of dynamic shared
// memory each: the smaller of the shared-memory and the register limit (80 registers a thread,
// as __launch_bounds__ fixes them).
int dec_ctas_per_sm(int threads, size_t smem) {
  struct SmemAttrs {
    size_t per_sm = 228 * 1024, reserved = 1024;
  };
  static const SmemAttrs attrs = [] {  // thread-safe one-time initialisation
    SmemAttrs a;
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) == cudaSuccess) a.per_sm = v;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrReservedSharedMemoryPerBlock, dev) == cudaSuccess) a.reserved = v;
    return a;
  }();
  const size_t by_smem = attrs.per_sm / (smem + attrs.reserved);
  const size_t by_regs = 65536 / (80 * (size_t)threads);
  return (int)std::min(by_smem, by_regs);
}

// The target stays in shared memory only if that costs no resident CTA (decided with Z off
// chip): the evaluation reads it once (into the environment matrix or the first state), so
// from L2 it costs one coalesced read per evaluation, while a shared copy of a six-qubit
// target (64 KB) would halve the CTAs an SM holds.  SQG_DECOMPOSE_TARGET=global|shared
// overrides the rule below six qubits.
bool dec_target_in_smem(const sqg_circuit* c, int cols) {
  if (c->n >= 6) return false;
  const char* tenv = getenv("SQG_DECOMPOSE_TARGET");
  if (tenv && std::string(tenv) == "global") return false;
  if (tenv && std::string(tenv) == "shared") return true;
  const int t = dec_threads(c);
  return dec_ctas_per_sm(t, dec_smem_layout(c, cols, true, false, false)) >=
         dec_ctas_per_sm(t, dec_smem_layout(c, cols, false, false, false));
}

size_t dec_smem_bytes(const sqg_circuit* c, int cols, bool z_in_smem, bool adam = false) {
  return dec_smem_layout(c, cols, dec_target_in_smem(c, cols), z_in_smem, adam);
}

constexpr size_t kDecSmemLimit = 110 * 1024;  // keep two CTAs per SM

// Per-instance BFGS matrices stay in shared memory only while they are small (<= 16 KB) and
// cost no resident CTA: beyond that, keeping them in the caller's workspace (L2-resident for
// the instances in flight) lets more instances share an SM, and the kernel is bound by FP64
// issue, not by L2 (six qubits, P = 36: 3 CTAs per SM instead of 2, +8.7%).
// SQG_DECOMPOSE_Z=global|shared overrides the rule.
bool z_in_shared(const sqg_circuit* c, int cols) {
  const char* zenv = getenv("SQG_DECOMPOSE_Z");
  if (zenv && std::string(zenv) == "global") return false;
  if (zenv && std::string(zenv) == "shared") return dec_smem_bytes(c, cols, true) <= 227 * 1024;
  const size_t with_z = dec_smem_bytes(c, cols, true);
  return (size_t)c->P * c->P * sizeof(double) <= 16 * 1024 && with_z <= kDecSmemLimit &&
         dec_ctas_per_sm(dec_threads(c), with_z) >= dec_ctas_per_sm(dec_threads(c), dec_smem_bytes(c, cols, false));
}

// The environment-matrix form costs 3 N^2 / 2 amplitude-pair updates per gate against
// 3 N cols / 2 for the state sweeps plus their per-gate inner products (the larger part
// at full width); it wins from about cols >= 3N/4.  SQG_DECOMPOSE_FORM=sweep|cyclic
// overrides the rule.
bool use_cyclic(const sqg_circuit* c, int cols) {
  const char* f = getenv("SQG_DECOMPOSE_FORM");
  if (f && std::string(f) == "sweep") return false;
  if (f && std::string(f) == "cyclic") return 2 * cols >= c->N;
  return 4 * cols >= 3 * c->N;
}

bool use_two_chains() {
  const char* f = getenv("SQG_DECOMPOSE_CHAINS");
  return !(f && std::string(f) == "1");
}

// Split gate h of the two-warp evaluation: minimises max(phase 1) + max(phase 2) of the
// two warps with the FP64 cost of each gate application (U3 14, one-parameter 8, CNOT/CZ
// about 1 for the exchange).
int two_chain_split(const sqg_circuit& c) {
  const int L = c.L;
  std::vector<double> w(L);
  for (int k = 0; k < L; k++) {
    const int t = c.h_gates[k].type;
    w[k] = t == G_U3 ? 14.0 : gate_param_num(t) == 1 ? 8.0 : 1.0;
  }
  int best = 1;
  double best_t = 1e300;
  for (int h = 1; h < L; h++) {
    double p1a = 0, p1b = 0, p2a = 0, p2b = 0;
    for (int k = 0; k < h; k++) p1a += w[k];
    for (int k = h + 1; k < L; k++) p1b += w[k];
    for (int k = 0; k < h; k++) p2a += w[k] + w[k + 1];
    for (int k = h; k < L - 1; k++) p2b += w[k] + w[k + 1];
    if (h == L - 1) p2b += w[h];
    const double t = std::max(p1a, p1b) + std::max(p2a, p2b);
    if (t < best_t) {
      best_t = t;
      best = h;
    }
  }
  return best;
}

// Kernel attributes and launch shared by the BFGS and ADAM entry points.
template <int OPT, int FORM, bool ZG>
int dec_launch_form(const sqg_circuit* c, const DecArgs& a, int batch, size_t smem, void* stream) {
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa = {};
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_decompose<OPT, FORM, ZG>);
  if (e == cudaSuccess && smem + fa.sharedSizeBytes > (size_t)optin)
    return set_error(SQG_ERR_UNSUPPORTED, "circuit too large for the batched decomposition kernel");
  // raised to the device maximum (less the kernel's static shared memory), never lowered:
  // the attribute is shared by all callers
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_decompose<OPT, FORM, ZG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             optin - (int)fa.sharedSizeBytes);
  if (e != cudaSuccess) {
    cudaGetLastError();  // leave no error behind for the next launch to report
    return set_error(SQG_ERR_CUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
  }
  k_decompose<OPT, FORM, ZG><<<batch, dec_threads(c), smem, (cudaStream_t)stream>>>(a);
  e = cudaGetLastError();
  return e == cudaSuccess ? SQG_OK : set_error(SQG_ERR_CUDA, std::string("k_decompose: ") + cudaGetErrorString(e));
}

template <int OPT, bool ZG>
int dec_launch_z(const sqg_circuit* c, const DecArgs& a, int batch, size_t smem, void* stream) {
  if (a.chains == 2) return dec_launch_form<OPT, kFormTwoChains, ZG>(c, a, batch, smem, stream);
  if (a.cyclic) return dec_launch_form<OPT, kFormCyclic, ZG>(c, a, batch, smem, stream);
  return dec_launch_form<OPT, kFormSweep, ZG>(c, a, batch, smem, stream);
}

// BFGS with its matrices in global slots runs the ZG kernels (L2-kept Z accesses).
template <int OPT>
int dec_launch(const sqg_circuit* c, const DecArgs& a, int batch, size_t smem, void* stream) {
  if constexpr (OPT == kBfgs) {
    if (!a.z_in_smem) return dec_launch_z<OPT, true>(c, a, batch, smem, stream);
  }
  return dec_launch_z<OPT, false>(c, a, batch, smem, stream);
}

template <int OPT, int FORM, bool ZG>
int dec_max_active_per_sm(const sqg_circuit* c, size_t smem) {
  int dev = 0, optin = 0, nb = 0;
  cudaFuncAttributes fa = {};
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  if (cudaFuncGetAttributes(&fa, k_decompose<OPT, FORM, ZG>) != cudaSuccess) return 0;
  if (smem + fa.sharedSizeBytes > (size_t)optin) return 0;
  if (cudaFuncSetAttribute(k_decompose<OPT, FORM, ZG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           optin - (int)fa.sharedSizeBytes) != cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_decompose<OPT, FORM, ZG>, dec_threads(c), smem) !=
      cudaSuccess)
    return 0;
  return nb;
}

// Slots for the BFGS matrices of a launch of `batch` instances with Z in global memory: the
// most CTAs of any evaluation form that the device can hold at once, at most one per
// instance (one per instance if the occupancy cannot be queried).
int dec_z_slots(const sqg_circuit* c, int cols, int batch) {
  const size_t smem = dec_smem_bytes(c, cols, false);
  int per_sm = std::max(dec_max_active_per_sm<kBfgs, kFormSweep, true>(c, smem),
                        std::max(dec_max_active_per_sm<kBfgs, kFormCyclic, true>(c, smem),
                                 dec_max_active_per_sm<kBfgs, kFormTwoChains, true>(c, smem)));
  cudaGetLastError();  // a failed query leaves no error behind
  int dev = 0, sms = 0;
  if (per_sm <= 0 || cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
    return batch;
  return (int)std::min<long long>(batch, (long long)per_sm * sms);
}

size_t round256(size_t x) { return (x + 255) / 256 * 256; }

// Bytes of the slot region: the matrices, then the occupancy bitmap.
size_t dec_z_bytes(const sqg_circuit* c, int slots) {
  return round256((size_t)slots * c->P * c->P * sizeof(double)) + round256((size_t)(slots + 31) / 32 * 4);
}

// Points a at the slot region at ws and clears its bitmap on the launch stream.
int dec_use_z_slots(DecArgs& a, const sqg_circuit* c, int slots, void* ws, void* stream) {
  a.zglob = (double*)ws;
  a.zslots = slots;
  a.zbits = (unsigned int*)((char*)ws + round256((size_t)slots * c->P * c->P * sizeof(double)));
  cudaError_t e = cudaMemsetAsync(a.zbits, 0, (size_t)(slots + 31) / 32 * 4, (cudaStream_t)stream);
  return e == cudaSuccess ? SQG_OK : set_error(SQG_ERR_CUDA, std::string("slot bitmap: ") + cudaGetErrorString(e));
}

// Evaluation form of the decomposition kernels for this circuit and target width.
void dec_eval_form(const sqg_circuit* c, int cols, int off, DecArgs& a) {
  a.has_lam = dec_needs_lam(c, cols) ? 1 : 0;
  a.tgt_in_smem = dec_target_in_smem(c, cols) ? 1 : 0;
  a.inv_cols = 1.0 / cols;
  a.cyclic = use_cyclic(c, cols) ? 1 : 0;
  a.chains = 1;
  a.split = 0;
  if (a.cyclic && cols == c->N && off == 0 && c->N * c->N / 2 <= 32 && c->L >= 2 && use_two_chains()) {
    a.chains = 2;
    a.split = two_chain_split(*c);
  }
}

// Checks batch gate lists against the circuit (the same gate types and parameter layout; only
// target and control qubits may differ, in range and distinct) and stages them at dst on the
// device, so that the kernel indexes in range.  Returns SQG_OK or the error status.
int stage_gate_lists(const sqg_circuit* c, const sqg_gate* gates, int batch, Gate* dst, void* stream) {
  const int L = c->L, n = c->n;
  std::vector<Gate> lists((size_t)batch * L);
  for (long long b = 0; b < batch; b++)
    for (int g = 0; g < L; g++) {
      const sqg_gate& in = gates[b * L + g];
      const Gate& t = c->h_gates[g];
      const bool ctl = gate_controlled(t.type);
      if (in.type != t.type || in.param_start != t.pstart)
        return set_error(SQG_ERR_INVALID_ARGUMENT, "gate list " + std::to_string(b) + " differs from the circuit's gate "
                                                       "types or parameter layout at gate " + std::to_string(g));
      if (in.target < 0 || in.target >= n || (ctl && (in.control < 0 || in.control >= n || in.control == in.target)))
        return set_error(SQG_ERR_INVALID_ARGUMENT, "gate list " + std::to_string(b) + ": qubit out of range at gate " +
                                                       std::to_string(g));
      lists[b * L + g] = Gate{in.type, in.target, ctl ? in.control : -1, in.param_start};
    }
  // pageable source: the call returns once the records are staged, so `lists` may go
  cudaError_t e = cudaMemcpyAsync(dst, lists.data(), sizeof(Gate) * lists.size(), cudaMemcpyHostToDevice,
                                  (cudaStream_t)stream);
  return e == cudaSuccess ? SQG_OK : set_error(SQG_ERR_CUDA, std::string("gate lists: ") + cudaGetErrorString(e));
}

}  // namespace

namespace sqg {

template <int FORM>
static int env_launch(const DecArgs& a, const double* theta, double* cost, double* grad, int threads, size_t smem,
                      cudaStream_t s) {
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa = {};
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_env_costgrad<FORM>);
  if (e == cudaSuccess && smem + fa.sharedSizeBytes > (size_t)optin)
    return set_error(SQG_ERR_UNSUPPORTED, "circuit too large for the environment-matrix evaluation");
  // the dynamic maximum leaves room for any static shared memory of the kernel
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_env_costgrad<FORM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             optin - (int)fa.sharedSizeBytes);
  if (e != cudaSuccess) {
    cudaGetLastError();  // leave no error behind for the next launch to report
    return set_error(SQG_ERR_CUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
  }
  k_env_costgrad<FORM><<<a.B, threads, smem, s>>>(a, theta, cost, grad);
  e = cudaGetLastError();
  return e == cudaSuccess ? SQG_OK : set_error(SQG_ERR_CUDA, std::string("k_env_costgrad: ") + cudaGetErrorString(e));
}

// Cost and gradient of B parameter vectors (B x P, contiguous) of a circuit of at most five
// qubits against targets with cols >= 3N/4 columns, one CTA per vector with the
// environment-matrix evaluation of the decomposition kernel.  Returns SQG_ERR_UNSUPPORTED
// (without launching) for shapes it does not take; sqg_cost_grad then uses the tile kernels.
int env_cost_grad(const sqg_circuit* c, const double* theta, int B, const void* target, int cols, long long tstride,
                  int off, int variant, double* cost, double* grad, void* stream) {
  const char* f = getenv("SQG_COSTGRAD_FORM");
  if (f && std::string(f) == "tile") return SQG_ERR_UNSUPPORTED;
  if (c->n > 5 || c->P == 0 || c->L == 0 || !grad || !use_cyclic(c, cols)) return SQG_ERR_UNSUPPORTED;
  const size_t smem = dec_smem_bytes(c, cols, false, false);
  if (smem > 100 * 1024) return SQG_ERR_UNSUPPORTED;
  DecArgs a = {};
  a.gates = c->d_gates;
  a.L = c->L; a.P = c->P; a.n = c->n; a.N = c->N; a.cols = cols;
  a.trace_offset = off;
  a.variant = variant;
  a.targets = (const double2*)target;
  a.tstride = tstride;
  a.B = B;
  dec_eval_form(c, cols, off, a);
  const int threads = dec_threads(c);
  cudaStream_t s = (cudaStream_t)stream;
  if (a.chains == 2) return env_launch<kFormTwoChains>(a, theta, cost, grad, threads, smem, s);
  return env_launch<kFormCyclic>(a, theta, cost, grad, threads, smem, s);
}

}  // namespace sqg

extern "C" {

size_t sqg_decompose_workspace_bytes(const sqg_circuit* c, int batch, int cols) {
  if (!c || batch <= 0 || cols <= 0) return 0;
  if (z_in_shared(c, cols)) return 256;
  return dec_z_bytes(c, dec_z_slots(c, cols, batch)) + 256;
}

int sqg_decompose_batched(const sqg_circuit* c, const void* targets, int cols, int batch, int trace_offset,
                          int cost_variant, double* x, double* cost, int* calls, int* iters, double tolerance,
                          int max_calls,
                          int max_outer, int iteration_loops, int stop_at_tolerance, unsigned long long seed,
                          void* workspace, size_t ws_bytes, void* stream) {
  if (!c || !targets || !x || !cost || !calls || batch <= 0 || batch > 0x7fffffff / 2 || cols <= 0 || cols > c->N)
    return set_error(SQG_ERR_INVALID_ARGUMENT, "bad circuit, batch, targets or outputs");
  if (c->P == 0) return set_error(SQG_ERR_INVALID_ARGUMENT, "the circuit has no free parameters");
  if (cost_variant != SQG_FROBENIUS_NORM && cost_variant != SQG_HILBERT_SCHMIDT_TEST && cost_variant != SQG_INFIDELITY)
    return set_error(SQG_ERR_UNSUPPORTED, "cost function variant not implemented by the engine");
  const int off = cost_variant == SQG_FROBENIUS_NORM ? trace_offset : 0;
  if (off < 0 || off + cols > c->N) return set_error(SQG_ERR_INVALID_ARGUMENT, "trace offset out of range");
  if (c->n > 6) return set_error(SQG_ERR_UNSUPPORTED, "batched decomposition keeps a whole target per CTA: qbit_num <= 6");
  if (max_calls < 1 || max_outer < 1 || iteration_loops < 1)
    return set_error(SQG_ERR_INVALID_ARGUMENT, "iteration limits must be positive");
  const bool zs = z_in_shared(c, cols);
  size_t smem = dec_smem_bytes(c, cols, zs);
  if (smem > 227 * 1024) return set_error(SQG_ERR_UNSUPPORTED, "circuit too large for the batched decomposition kernel");
  const int slots = zs ? 0 : dec_z_slots(c, cols, batch);
  if (!zs && (!workspace || ((size_t)workspace & 255) || ws_bytes < dec_z_bytes(c, slots)))
    return set_error(SQG_ERR_WORKSPACE, "workspace too small or not 256-byte aligned for the BFGS matrices: need " +
                                            std::to_string(dec_z_bytes(c, slots)));
  DecArgs a = {};
  a.gates = c->d_gates;
  a.L = c->L; a.P = c->P; a.n = c->n; a.N = c->N; a.cols = cols;
  a.trace_offset = off;
  a.variant = cost_variant;
  a.targets = (const double2*)targets;
  a.tstride = (long long)c->N * cols;
  a.x = x; a.cost = cost; a.calls = calls; a.iters = iters;
  a.B = batch;
  a.tol = tolerance;
  a.max_calls = max_calls; a.max_outer = max_outer; a.loops = iteration_loops;
  a.early_stop = stop_at_tolerance;
  a.seed = seed;
  a.z_in_smem = zs ? 1 : 0;
  if (!zs)
    if (int st = dec_use_z_slots(a, c, slots, workspace, stream)) return st;
  dec_eval_form(c, cols, off, a);
  return dec_launch<kBfgs>(c, a, batch, smem, stream);
}


size_t sqg_decompose_structures_workspace_bytes(const sqg_circuit* c, int batch, int cols) {
  if (!c || batch <= 0 || cols <= 0) return 0;
  const size_t z = z_in_shared(c, cols) ? 0 : dec_z_bytes(c, dec_z_slots(c, cols, batch));
  return z + (size_t)batch * std::max(c->L, 1) * sizeof(Gate) + 256;
}

int sqg_decompose_structures(const sqg_circuit* c, const sqg_gate* gates, const void* targets,
                             long long target_stride, int cols, int batch, int trace_offset, int cost_variant,
                             double* x, double* cost, int* calls, int* iters, double tolerance, int max_calls,
                             int max_outer, int iteration_loops, int stop_at_tolerance, unsigned long long seed,
                             void* workspace, size_t ws_bytes, void* stream) {
  if (!c || !gates || !targets || !x || !cost || !calls || batch <= 0 || batch > 0x7fffffff / 2 || cols <= 0 ||
      cols > c->N)
    return set_error(SQG_ERR_INVALID_ARGUMENT, "bad circuit, gate lists, batch, targets or outputs");
  if (c->P == 0) return set_error(SQG_ERR_INVALID_ARGUMENT, "the circuit has no free parameters");
  if (cost_variant != SQG_FROBENIUS_NORM && cost_variant != SQG_HILBERT_SCHMIDT_TEST && cost_variant != SQG_INFIDELITY)
    return set_error(SQG_ERR_UNSUPPORTED, "cost function variant not implemented by the engine");
  const int off = cost_variant == SQG_FROBENIUS_NORM ? trace_offset : 0;
  if (off < 0 || off + cols > c->N) return set_error(SQG_ERR_INVALID_ARGUMENT, "trace offset out of range");
  if (c->n > 6) return set_error(SQG_ERR_UNSUPPORTED, "batched decomposition keeps a whole target per CTA: qbit_num <= 6");
  if (max_calls < 1 || max_outer < 1 || iteration_loops < 1)
    return set_error(SQG_ERR_INVALID_ARGUMENT, "iteration limits must be positive");
  if (target_stride != 0 && target_stride < (long long)c->N * cols)
    return set_error(SQG_ERR_INVALID_ARGUMENT, "target stride must be 0 (one shared target) or at least rows * cols");
  const bool zs = z_in_shared(c, cols);
  const size_t smem = dec_smem_bytes(c, cols, zs);
  if (smem > 227 * 1024) return set_error(SQG_ERR_UNSUPPORTED, "circuit too large for the batched decomposition kernel");
  const size_t need = sqg_decompose_structures_workspace_bytes(c, batch, cols);
  if (!workspace || ws_bytes < need || ((size_t)workspace & 255))
    return set_error(SQG_ERR_WORKSPACE, "workspace too small or not 256-byte aligned: need " + std::to_string(need));
  const int L = c->L, n = c->n;
  const int slots = zs ? 0 : dec_z_slots(c, cols, batch);
  const size_t zbytes = zs ? 0 : dec_z_bytes(c, slots);
  Gate* dgates = (Gate*)((char*)workspace + zbytes);
  if (int st = stage_gate_lists(c, gates, batch, dgates, stream)) return st;
  DecArgs a = {};
  a.gates = dgates;
  a.gstride = L;
  a.L = L; a.P = c->P; a.n = n; a.N = c->N; a.cols = cols;
  a.trace_offset = off;
  a.variant = cost_variant;
  a.targets = (const double2*)targets;
  a.tstride = target_stride;
  a.x = x; a.cost = cost; a.calls = calls; a.iters = iters;
  a.B = batch;
  a.tol = tolerance;
  a.max_calls = max_calls; a.max_outer = max_outer; a.loops = iteration_loops;
  a.early_stop = stop_at_tolerance;
  a.seed = seed;
  a.z_in_smem = zs ? 1 : 0;
  if (!zs)
    if (int st = dec_use_z_slots(a, c, slots, workspace, stream)) return st;
  dec_eval_form(c, cols, off, a);
  return dec_launch<kBfgs>(c, a, batch, smem, stream);
}

int sqg_decompose_batched_adam(const sqg_circuit* c, const void* targets, int cols, int batch, int trace_offset,
                               int cost_variant, double* x, double* cost, int* evals, int* shifts, double tolerance,
                               int max_iters, double eta, int adaptive_eta, int random_shift_count_max,
                               long long randomization_threshold, int max_outer, unsigned long long seed,
                               void* stream) {
  if (!c || !targets || !x || !cost || !evals || batch <= 0 || batch > 0x7fffffff / 2 || cols <= 0 || cols > c->N)
    return set_error(SQG_ERR_INVALID_ARGUMENT, "bad circuit, batch, targets or outputs");
  if (c->P == 0) return set_error(SQG_ERR_INVALID_ARGUMENT, "the circuit has no free parameters");
  if (cost_variant != SQG_FROBENIUS_NORM && cost_variant != SQG_HILBERT_SCHMIDT_TEST && cost_variant != SQG_INFIDELITY)
    return set_error(SQG_ERR_UNSUPPORTED, "cost function variant not implemented by the engine");
  const int off = cost_variant == SQG_FROBENIUS_NORM ? trace_offset : 0;
  if (off < 0 || off + cols > c->N) return set_error(SQG_ERR_INVALID_ARGUMENT, "trace offset out of range");
  if (c->n > 6) return set_error(SQG_ERR_UNSUPPORTED, "batched decomposition keeps a whole target per CTA: qbit_num <= 6");
  if (max_iters < 1 || max_outer < 1 || random_shift_count_max < 0 || randomization_threshold < 0)
    return set_error(SQG_ERR_INVALID_ARGUMENT, "iteration limits must be positive");
  const size_t smem = dec_smem_bytes(c, cols, false, true);
  if (smem > 227 * 1024) return set_error(SQG_ERR_UNSUPPORTED, "circuit too large for the batched decomposition kernel");
  DecArgs a = {};
  a.gates = c->d_gates;
  a.L = c->L; a.P = c->P; a.n = c->n; a.N = c->N; a.cols = cols;
  a.trace_offset = off;
  a.variant = cost_variant;
  a.targets = (const double2*)targets;
  a.tstride = (long long)c->N * cols;
  a.x = x; a.cost = cost; a.calls = evals; a.iters = shifts;
  a.B = batch;
  a.tol = tolerance;
  a.max_calls = max_iters; a.max_outer = max_outer; a.loops = 1;
  a.early_stop = 1;
  a.seed = seed;
  a.zglob = nullptr;
  a.z_in_smem = 0;
  a.eta = eta;
  a.adaptive_eta = adaptive_eta ? 1 : 0;
  a.shift_max = random_shift_count_max;
  a.rand_thr = randomization_threshold;
  dec_eval_form(c, cols, off, a);
  return dec_launch<kAdam>(c, a, batch, smem, stream);
}

size_t sqg_decompose_structures_adam_workspace_bytes(const sqg_circuit* c, int batch) {
  if (!c || batch <= 0) return 0;
  return (size_t)batch * std::max(c->L, 1) * sizeof(Gate) + 256;
}

int sqg_decompose_structures_adam(const sqg_circuit* c, const sqg_gate* gates, const void* targets,
                                  long long target_stride, int cols, int batch, int trace_offset, int cost_variant,
                                  double* x, double* cost, int* evals, int* shifts, double tolerance, int max_iters,
                                  double eta, int adaptive_eta, int random_shift_count_max,
                                  long long randomization_threshold, int max_outer, unsigned long long seed,
                                  void* workspace, size_t ws_bytes, void* stream) {
  if (!c || !gates || !targets || !x || !cost || !evals || batch <= 0 || batch > 0x7fffffff / 2 || cols <= 0 ||
      cols > c->N)
    return set_error(SQG_ERR_INVALID_ARGUMENT, "bad circuit, gate lists, batch, targets or outputs");
  if (c->P == 0) return set_error(SQG_ERR_INVALID_ARGUMENT, "the circuit has no free parameters");
  if (cost_variant != SQG_FROBENIUS_NORM && cost_variant != SQG_HILBERT_SCHMIDT_TEST && cost_variant != SQG_INFIDELITY)
    return set_error(SQG_ERR_UNSUPPORTED, "cost function variant not implemented by the engine");
  const int off = cost_variant == SQG_FROBENIUS_NORM ? trace_offset : 0;
  if (off < 0 || off + cols > c->N) return set_error(SQG_ERR_INVALID_ARGUMENT, "trace offset out of range");
  if (c->n > 6) return set_error(SQG_ERR_UNSUPPORTED, "batched decomposition keeps a whole target per CTA: qbit_num <= 6");
  if (max_iters < 1 || max_outer < 1 || random_shift_count_max < 0 || randomization_threshold < 0)
    return set_error(SQG_ERR_INVALID_ARGUMENT, "iteration limits must be positive");
  if (target_stride != 0 && target_stride < (long long)c->N * cols)
    return set_error(SQG_ERR_INVALID_ARGUMENT, "target stride must be 0 (one shared target) or at least rows * cols");
  const size_t smem = dec_smem_bytes(c, cols, false, true);
  if (smem > 227 * 1024) return set_error(SQG_ERR_UNSUPPORTED, "circuit too large for the batched decomposition kernel");
  const size_t need = sqg_decompose_structures_adam_workspace_bytes(c, batch);
  if (!workspace || ws_bytes < need || ((size_t)workspace & 255))
    return set_error(SQG_ERR_WORKSPACE, "workspace too small or not 256-byte aligned: need " + std::to_string(need));
  Gate* dgates = (Gate*)workspace;
  if (int st = stage_gate_lists(c, gates, batch, dgates, stream)) return st;
  DecArgs a = {};
  a.gates = dgates;
  a.gstride = c->L;
  a.L = c->L; a.P = c->P; a.n = c->n; a.N = c->N; a.cols = cols;
  a.trace_offset = off;
  a.variant = cost_variant;
  a.targets = (const double2*)targets;
  a.tstride = target_stride;
  a.x = x; a.cost = cost; a.calls = evals; a.iters = shifts;
  a.B = batch;
  a.tol = tolerance;
  a.max_calls = max_iters; a.max_outer = max_outer; a.loops = 1;
  a.early_stop = 1;
  a.seed = seed;
  a.zglob = nullptr;
  a.z_in_smem = 0;
  a.eta = eta;
  a.adaptive_eta = adaptive_eta ? 1 : 0;
  a.shift_max = random_shift_count_max;
  a.rand_thr = randomization_threshold;
  dec_eval_form(c, cols, off, a);
  return dec_launch<kAdam>(c, a, batch, smem, stream);
}

}  // extern "C"
