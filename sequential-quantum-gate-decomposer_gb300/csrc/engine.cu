// GB300 engine for the SQUANDER decomposition hot path: cost and adjoint gradient of a
// parametric circuit applied to a 2^n x cols complex128 target, plus forward/right
// application and the combined-unitary parity API.  Entry points are declared in
// include/sqg.h.
//
// Design (GB300-first, one GPU):
//  * Column tiles.  Gates mix rows only, so every column of U^dagger is an independent
//    state vector.  A CTA loads a tile of TC columns into shared memory (column-major:
//    each column contiguous), applies ALL L gates there, and reads HBM once.  The whole
//    circuit is fused, whatever qubits it touches (n <= 13 fits a column in 128 KB).
//  * Adjoint gradient per column: psi = C u_j is uncomputed gate by gate with G^dagger
//    while the co-state lambda (starting at e_{j+offset}) is propagated with G^dagger;
//    for each parametric gate the 2x2 overlap R_ab = sum conj(lambda_a) psi_b is reduced
//    over the tile and contracted with the derivative kernels.  O(L) passes in shared
//    memory replace the reference's (P+1) dense derivative matrices.
//  * FP64 is the binding resource on GB300, so the update rules (gates.cuh) minimise FP64
//    instructions and everything else (index math, exchanges, sign flips) is integer work.
//  * Deterministic reductions: per-tile partial traces go to the caller's workspace and
//    are summed in a fixed order by a second kernel.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/sqg.h"
#include "gates.cuh"
#include "handle.h"
#include "tile.cuh"
#include "tilekern.cuh"

using namespace sqg;

namespace {
thread_local std::string g_last_error;
}  // namespace

int sqg::set_error(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}

namespace {

int fail(int status, const std::string& msg) { return sqg::set_error(status, msg); }

int cuda_status(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return SQG_OK;
  g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
  return SQG_ERR_CUDA;
}

constexpr int kMaxThreads = 256;
constexpr size_t kSmemBudgetFwd = 100 * 1024;   // column tile budget, forward only (n = 12: one column, 3 CTAs/SM)
constexpr size_t kSmemBudgetGrad = 100 * 1024;  // psi + lambda tiles

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// -------------------------------------------------------------------------------------
// Gate-matrix preparation: one thread per (instance, gate).  Each parameter belongs to
// exactly one gate, so sin/cos of each stored parameter is evaluated once
// (Gates_block.cpp:269-279 evaluates them the same way, per parameter).
// -------------------------------------------------------------------------------------
__global__ void k_prep(const Gate* __restrict__ gates, int L, int P, const double* __restrict__ theta,
                       long long theta_stride, int B, GateMat* __restrict__ gm, double2* __restrict__ sc) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  int b = blockIdx.y;
  if (g >= L || b >= B) return;
  Gate gt = gates[g];
  const double* th = theta + (long long)b * theta_stride + gt.pstart;
  GateMat m;
  m.u[0] = m.u[1] = m.u[2] = m.u[3] = make_double2(0.0, 0.0);
  double2* scb = sc + (long long)b * P + gt.pstart;
  if (gt.type == G_U3) {
    double st, ct, sp, cp, sl, cl;
    sincos(th[0], &st, &ct);
    sincos(th[1], &sp, &cp);
    sincos(th[2], &sl, &cl);
    scb[0] = make_double2(st, ct);
    scb[1] = make_double2(sp, cp);
    scb[2] = make_double2(sl, cl);
    double spl = sp * cl + cp * sl, cpl = cp * cl - sp * sl;
    // gate_kernel_templates.h:509-521
    m.u[0] = make_double2(ct, 0.0);
    m.u[1] = make_double2(-st * cl, -st * sl);
    m.u[2] = make_double2(st * cp, st * sp);
    m.u[3] = make_double2(ct * cpl, ct * spl);
  } else if (gate_param_num(gt.type) == 1) {
    double s, c;
    sincos(th[0], &s, &c);
    scb[0] = make_double2(s, c);
    m.u[0] = make_double2(c, s);
  }
  gm[(long long)b * L + g] = m;
}

template <bool WRITE_BACK, bool TRACE>
__global__ void __launch_bounds__(kMaxThreads) k_tile_forward(TileArgs a) {
  extern __shared__ double2 smem[];
  tile_forward_body<WRITE_BACK, TRACE>(a, blockIdx.y, blockIdx.x, smem);
}

__global__ void __launch_bounds__(kMaxThreads) k_tile_adjoint(TileArgs a) {
  extern __shared__ double2 smem[];
  tile_adjoint_body(a, blockIdx.y, blockIdx.x, smem);
}

// Sums the per-tile partials in a fixed order and applies the cost-variant epilogue of
// the reference (Optimization_Interface.cpp:677-735 for the cost, :1397-1458 for the
// gradient components).
__global__ void k_finish(const double2* __restrict__ ws_tr, const double2* __restrict__ ws_gr, int tiles, int P,
                         int cols, int variant, double* __restrict__ cost, double* __restrict__ grad) {
  const int b = blockIdx.x;
  double2 tr = make_double2(0.0, 0.0);
  for (int t = 0; t < tiles; t++) {
    double2 v = ws_tr[(long long)b * tiles + t];
    tr.x += v.x;
    tr.y += v.y;
  }
  if (blockIdx.y == 0 && threadIdx.x == 0) {
    double f;
    if (variant == SQG_FROBENIUS_NORM) {
      f = 1.0 - tr.x / cols;
    } else if (variant == SQG_HILBERT_SCHMIDT_TEST) {
      double d = 1.0 / cols;
      f = 1.0 - d * d * (tr.x * tr.x + tr.y * tr.y);
    } else {
      double d = cols;
      f = 1.0 - ((tr.x * tr.x + tr.y * tr.y) / d + 1) / (d + 1);
    }
    cost[b] = f;
  }
  if (!grad) return;
  const int p = blockIdx.y * blockDim.x + threadIdx.x;
  if (p >= P) return;
  double2 dt = make_double2(0.0, 0.0);
  for (int t = 0; t < tiles; t++) {
    double2 v = ws_gr[((long long)b * tiles + t) * P + p];
    dt.x += v.x;
    dt.y += v.y;
  }
  double gv;
  if (variant == SQG_FROBENIUS_NORM) {
    gv = (1.0 - dt.x / cols) - 1.0;
  } else if (variant == SQG_HILBERT_SCHMIDT_TEST) {
    double d = 1.0 / cols;
    gv = -2.0 * d * d * tr.x * dt.x - 2.0 * d * d * tr.y * dt.y;
  } else {
    double d = cols;
    gv = -2.0 / d / (d + 1) * tr.x * dt.x - 2.0 / d / (d + 1) * tr.y * dt.y;
  }
  grad[(long long)b * P + p] = gv;
}

// -------------------------------------------------------------------------------------
// One pass over an HBM-resident matrix per gate (unfused application and the
// combined-unitary parity API).  Thread = one amplitude pair x one column; consecutive
// threads take consecutive columns, so every access is a coalesced 16-byte load.
// deriv_k < 0: forward gate from gm; deriv_k >= 0: derivative kernel of parameter
// deriv_k built from the stored sin/cos, with the pairs whose control bit is clear
// zeroed (apply_kernel_to_input.cpp:93-97).
// -------------------------------------------------------------------------------------
__global__ void k_gate_hbm(double2* __restrict__ mtx, long long bstride, long long rstride, int cols, int logN,
                           Gate gt, const GateMat* __restrict__ gmp, const double2* __restrict__ scp, int deriv_k,
                           int nmat) {
  const bool ctrl = gate_controlled(gt.type);
  const bool deriv = deriv_k >= 0;
  const int lognp = (!deriv && ctrl) ? logN - 2 : logN - 1;
  const long long items = (long long)cols << lognp;
  const int step = 1 << gt.target;
  PairOp op;
  double2 D[4];
  if (deriv) {
    deriv_kernel(gt.type, scp + gt.pstart, deriv_k, D);
  } else {
    op = make_op(gt.type, *gmp, ORIENT_FWD);
  }
  // items < 2^31 (at most 2^29 pairs of a 30-qubit state, 2^12 x 2^13 pairs of a matrix);
  // a power-of-two column count splits an item with a shift instead of a division
  const int logc = (__popc(cols) == 1) ? __ffs(cols) - 1 : -1;
  for (int b = blockIdx.y; b < nmat; b += gridDim.y) {
    double2* base = mtx + (long long)b * bstride;
    for (unsigned it = blockIdx.x * blockDim.x + threadIdx.x; it < (unsigned)items; it += gridDim.x * blockDim.x) {
      int p, c;
      if (logc >= 0) {
        p = (int)(it >> logc);
        c = (int)(it & (unsigned)(cols - 1));
      } else {
        p = (int)(it / (unsigned)cols);
        c = (int)(it - (unsigned)p * (unsigned)cols);
      }
      int i;
      bool active = true;
      if (!deriv) {
        i = ctrl ? pair_index2(p, gt.target, gt.control) : pair_index1(p, gt.target);
      } else {
        i = pair_index1(p, gt.target);
        active = !ctrl || ((i >> gt.control) & 1);
      }
      double2* px = base + (long long)i * rstride + c;
      double2* py = base + (long long)(i + step) * rstride + c;
      if (!active) {
        *px = make_double2(0.0, 0.0);
        *py = make_double2(0.0, 0.0);
        continue;
      }
      double2 x = *px, y = *py;
      if (!deriv) {
        apply_op(op, x, y);
      } else {
        double2 nx, ny;
        nx.x = D[0].x * x.x - D[0].y * x.y + D[1].x * y.x - D[1].y * y.y;
        nx.y = D[0].x * x.y + D[0].y * x.x + D[1].x * y.y + D[1].y * y.x;
        ny.x = D[2].x * x.x - D[2].y * x.y + D[3].x * y.x - D[3].y * y.y;
        ny.y = D[2].x * x.y + D[2].y * x.x + D[3].x * y.y + D[3].y * y.x;
        x = nx;
        y = ny;
      }
      *px = x;
      *py = y;
    }
  }
}

// CNOT and CZ on an HBM-resident matrix or state (one pass per gate, no FP64 instruction, so
// the pass is bound by HBM alone).  An item is one element of a touched row; consecutive
// threads take consecutive elements, so every load and store instruction of a warp covers
// 512 contiguous bytes.  A thread handles 4 items a grid-stride apart and issues all their loads
// before its stores (8 loads in flight for CNOT).  CNOT exchanges the two rows of every pair
// whose control bit is set (half of the rows); CZ negates, by flipping sign bits, only the
// target = 1 row of those pairs (a quarter of the rows) and reads nothing else.
// `col_shift` = log2(cols) when cols is a power of two, else -1.
template <int KIND>  // 0: CNOT, 1: CZ
__global__ void __launch_bounds__(256) k_perm_hbm(double2* __restrict__ mtx, long long rstride, int cols,
                                                  int col_shift, long long items, int target, int control) {
  constexpr int U = 4;
  const int step = 1 << target;
  const unsigned long long sign = 0x8000000000000000ULL;
  const long long T = (long long)gridDim.x * blockDim.x;
  for (long long it0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; it0 < items; it0 += U * T) {
    double2* px[U];
    double2* py[U];
    double2 a[U], b[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const long long it = it0 + k * T;
      px[k] = py[k] = nullptr;
      if (it < items) {
        const int pr = col_shift >= 0 ? (int)(it >> col_shift) : (int)(it / cols);
        const int c = (int)(it - (long long)pr * cols);
        const int i = pair_index2(pr, target, control);
        px[k] = mtx + (long long)i * rstride + c;
        py[k] = mtx + (long long)(i + step) * rstride + c;
      }
    }
#pragma unroll
    for (int k = 0; k < U; ++k) {
      if (py[k]) {
        b[k] = *py[k];
        if (KIND == 0) a[k] = *px[k];
      }
    }
#pragma unroll
    for (int k = 0; k < U; ++k) {
      if (!py[k]) continue;
      if (KIND == 0) {
        *px[k] = b[k];
        *py[k] = a[k];
      } else {
        *py[k] = make_double2(__longlong_as_double(__double_as_longlong(b[k].x) ^ (long long)sign),
                              __longlong_as_double(__double_as_longlong(b[k].y) ^ (long long)sign));
      }
    }
  }
}

int hbm_blocks(long long items) { return (int)std::min<long long>((items + 255) / 256, 152LL * 16); }

// ---- launch helpers ------------------------------------------------------------------
struct TilePlan {
  int TC, tiles, threads;
  size_t smem;
};

int choose_threads(int tc, int N, bool grad) {
  int items = tc * (N / 2);
  int t = std::min(kMaxThreads, std::max(32, (items + 31) / 32 * 32));
  (void)grad;
  return t;
}

int device_sms() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 1;
  return std::max(sms, 1);
}

// Column tiles of a launch over B instances of `cols` columns.  A tile holds as many columns
// as the shared-memory budget takes (a power of two); when the whole launch would then not
// give every SM two CTAs (small batches: a single decomposition's evaluation), tiles are
// narrowed down to one column each, so the FP64 work of one instance spreads over the GPU.
TilePlan plan_tiles(int N, int cols, bool grad, int B = 0) {
  const size_t per = (size_t)N * sizeof(double2) * (grad ? 2 : 1);
  size_t budget = grad ? kSmemBudgetGrad : kSmemBudgetFwd;
  int tc = (int)std::max<size_t>(1, budget / per);
  // prefer powers of two, never more than the vectors available
  int p2 = 1;
  while (p2 * 2 <= tc) p2 *= 2;
  tc = std::min(p2, cols);
  if (B > 0) {
    const long long want = 2LL * device_sms();
    while (tc > 1 && (long long)B * ((cols + tc - 1) / tc) < want) tc >>= 1;
  }
  TilePlan pl;
  pl.TC = tc;
  pl.tiles = (cols + tc - 1) / tc;
  pl.threads = choose_threads(tc, N, grad);
  pl.smem = tile_smem_bytes(tc, N, grad);
  return pl;
}

// Raises a kernel's dynamic shared memory limit to the device's opt-in maximum (never
// lowers it: the attribute is shared by every caller of the kernel).
template <typename K>
int set_smem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kernel);
    const size_t dyn_max = e == cudaSuccess ? (size_t)optin - fa.sharedSizeBytes : 0;  // minus static shared memory
    if (e == cudaSuccess && bytes > dyn_max) return fail(SQG_ERR_UNSUPPORTED, "tile exceeds shared memory");
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_max);
    if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute");
  }
  return SQG_OK;
}

struct PrepLayout {
  size_t gm_off, sc_off, mg_off, end;
};
PrepLayout prep_layout(const sqg_circuit* c, int B, size_t start) {
  PrepLayout l;
  l.gm_off = align_up(start, 256);
  l.sc_off = align_up(l.gm_off + (size_t)B * std::max(c->L, 1) * sizeof(GateMat), 256);
  l.mg_off = align_up(l.sc_off + (size_t)B * std::max(c->P, 1) * sizeof(double2), 256);
  l.end = align_up(l.mg_off + (size_t)B * c->Lm * sizeof(GateMat), 256);
  return l;
}

// Full 2x2 matrix of a single-qubit gate from its GateMat (k_prep's storage: U3 whole, the
// one-parameter gates as (cos, sin) in u[0]).
__device__ __forceinline__ void full_matrix(int type, const GateMat& m, double2 u[4]) {
  const double c = m.u[0].x, s = m.u[0].y;
  if (type == G_U3) {
    u[0] = m.u[0]; u[1] = m.u[1]; u[2] = m.u[2]; u[3] = m.u[3];
  } else if (type == G_RY) {
    u[0] = make_double2(c, 0.0); u[1] = make_double2(dneg(s), 0.0);
    u[2] = make_double2(s, 0.0); u[3] = make_double2(c, 0.0);
  } else if (type == G_RX) {
    u[0] = make_double2(c, 0.0); u[1] = make_double2(0.0, dneg(s));
    u[2] = make_double2(0.0, dneg(s)); u[3] = make_double2(c, 0.0);
  } else {  // G_RZ
    u[0] = make_double2(c, dneg(s)); u[1] = make_double2(0.0, 0.0);
    u[2] = make_double2(0.0, 0.0); u[3] = make_double2(c, s);
  }
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}

// Gate matrices of the merged forward plan, one thread per (instance, merged gate): a kept
// gate copies its matrix, a merged run multiplies its members' matrices in circuit order
// (M = G_k ... G_1).
__global__ void k_merge(const Gate* __restrict__ gates, const GateMat* __restrict__ gm, int L,
                        const Gate* __restrict__ mgates, const int* __restrict__ mfirst,
                        const int* __restrict__ members, int Lm, GateMat* __restrict__ out) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (m >= Lm) return;
  const GateMat* g = gm + (long long)b * L;
  const int f = mfirst[m], e = mfirst[m + 1];
  GateMat r;
  if (mgates[m].type != G_GEN) {
    r = g[members[f]];
  } else {
    double2 M[4];
    full_matrix(gates[members[f]].type, g[members[f]], M);
    for (int k = f + 1; k < e; k++) {
      double2 G[4], R[4];
      full_matrix(gates[members[k]].type, g[members[k]], G);
      R[0] = cmul(G[0], M[0]); R[0].x += cmul(G[1], M[2]).x; R[0].y += cmul(G[1], M[2]).y;
      R[1] = cmul(G[0], M[1]); R[1].x += cmul(G[1], M[3]).x; R[1].y += cmul(G[1], M[3]).y;
      R[2] = cmul(G[2], M[0]); R[2].x += cmul(G[3], M[2]).x; R[2].y += cmul(G[3], M[2]).y;
      R[3] = cmul(G[2], M[1]); R[3].x += cmul(G[3], M[3]).x; R[3].y += cmul(G[3], M[3]).y;
      M[0] = R[0]; M[1] = R[1]; M[2] = R[2]; M[3] = R[3];
    }
    r.u[0] = M[0]; r.u[1] = M[1]; r.u[2] = M[2]; r.u[3] = M[3];
  }
  out[(long long)b * Lm + m] = r;
}

// Forward gate list and matrices of a tile launch: the merged plan when the circuit has one
// (its matrices computed into the workspace at prep.mg_off), else the gates themselves.
int forward_plan(const sqg_circuit* c, const PrepLayout& prep, char* ws, int B, const GateMat* gm, TileArgs& a,
                 cudaStream_t st) {
  if (c->Lm == 0) {
    a.gates = c->d_gates;
    a.L = c->L;
    a.gm = gm;
    return SQG_OK;
  }
  GateMat* mg = (GateMat*)(ws + prep.mg_off);
  k_merge<<<dim3((c->Lm + 127) / 128, B), 128, 0, st>>>(c->d_gates, gm, c->L, c->d_mgates, c->d_mfirst,
                                                         c->d_mmembers, c->Lm, mg);
  a.gates = c->d_mgates;
  a.L = c->Lm;
  a.gm = mg;
  return cuda_status(cudaGetLastError(), "k_merge");
}

struct EvalLayout {
  PrepLayout prep;
  size_t tr_off, gr_off, ck_off, end;
  TilePlan plan;
  int nck;
};
EvalLayout eval_layout(const sqg_circuit* c, int B, int cols, bool grad, int ckpt_interval) {
  EvalLayout l;
  l.prep = prep_layout(c, B, 0);
  l.plan = plan_tiles(c->N, cols, grad, B);
  l.tr_off = l.prep.end;
  l.gr_off = align_up(l.tr_off + (size_t)B * l.plan.tiles * sizeof(double2), 256);
  size_t gr_bytes = grad ? (size_t)B * l.plan.tiles * std::max(c->P, 1) * sizeof(double2) : 0;
  l.ck_off = align_up(l.gr_off + gr_bytes, 256);
  l.nck = 0;
  if (grad && ckpt_interval > 0) l.nck = c->L / ckpt_interval;
  size_t ck_bytes = (size_t)B * l.plan.tiles * l.nck * (size_t)l.plan.TC * c->N * sizeof(double2);
  l.end = align_up(l.ck_off + ck_bytes, 256);
  return l;
}

int launch_prep(const sqg_circuit* c, const double* theta, long long theta_stride, int B, GateMat* gm, double2* sc,
                cudaStream_t st) {
  if (c->L == 0) return SQG_OK;
  dim3 grid((c->L + 127) / 128, B);
  k_prep<<<grid, 128, 0, st>>>(c->d_gates, c->L, c->P, theta, theta_stride, B, gm, sc);
  return cuda_status(cudaGetLastError(), "k_prep");
}

// Matrix entry points hold whole columns in shared memory: qbit_num <= kMatrixQubits.
constexpr int kMatrixQubits = 13;

int check_circuit(const sqg_circuit* c, int max_n = kMatrixQubits) {
  if (!c) return fail(SQG_ERR_INVALID_ARGUMENT, "null circuit handle");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != c->device) return fail(SQG_ERR_INVALID_ARGUMENT, "circuit handle belongs to another device");
  if (c->n > max_n)
    return fail(SQG_ERR_UNSUPPORTED, "this entry point supports qbit_num <= " + std::to_string(max_n) +
                                         " (state vectors up to 30 qubits: sqg_apply_state)");
  return SQG_OK;
}

// ---- state vectors ---------------------------------------------------------------------
constexpr int kStateQubits = 30;   // largest register of sqg_apply_state (2^30 amplitudes, 16 GiB)
constexpr int kStateK = 12;        // qubits per chunk: 4096 amplitudes, 64 KB of shared memory
constexpr int kStateLow = 5;       // the lowest qubits belong to every chunk (512-byte coalesced runs)
constexpr int kStateThreads = 256;

// Groups the gates into blocks: a block grows while the qubits it touches, together with the
// lowest kStateLow ones, number at most K; each block is one pass over the state.  With
// partition ends (`cuts`, the gate index after each partition) a block grows by whole
// partitions and breaks only between them, unless one partition alone exceeds the chunk (it
// is then split gate by gate).  Fills the chunk with further qubits (lowest first), maps every
// gate of the block to chunk-local qubit positions and tabulates the global offsets of the
// chunk's high local bits and the qubits that number the chunks.
int build_state_plan(sqg_circuit* c, const std::vector<int>& cuts = {}) {
  const int n = c->n, K = std::min(n, kStateK), low = std::min(K, kStateLow);
  c->sK = K;
  std::vector<Gate> lg(c->h_gates);
  std::vector<int> hitab, inact;
  std::vector<int> inA(n, 0);
  auto close_block = [&](int g0, int g1) {
    std::vector<int> A;
    for (int q = 0; q < n; q++)
      if (q < low || inA[q]) A.push_back(q);
    for (int q = 0; q < n && (int)A.size() < K; q++)
      if (!(q < low || inA[q])) {
        A.push_back(q);
        inA[q] = 1;
      }
    std::sort(A.begin(), A.end());
    std::vector<int> loc(n, -1);
    for (int j = 0; j < (int)A.size(); j++) loc[A[j]] = j;
    for (int g = g0; g < g1; g++) {
      lg[g].target = loc[c->h_gates[g].target];
      if (gate_controlled(c->h_gates[g].type)) lg[g].control = loc[c->h_gates[g].control];
    }
    const int hb = K - low;
    for (int h = 0; h < 128; h++) {
      int off = 0;
      if (h < (1 << hb))
        for (int j = 0; j < hb; j++)
          if ((h >> j) & 1) off |= 1 << A[low + j];
      hitab.push_back(off);
    }
    int k = 0;
    for (int q = 0; q < n; q++)
      if (loc[q] < 0) {
        inact.push_back(q);
        k++;
      }
    for (; k < 32; k++) inact.push_back(0);
    c->sblocks.push_back({g0, g1});
    std::fill(inA.begin(), inA.end(), 0);
  };
  int g0 = 0, used = 0;
  auto take_gate = [&](int g) {  // gate by gate: break wherever the chunk would overflow
    const Gate& gt = c->h_gates[g];
    int add = 0;
    int qs[2] = {gt.target, gate_controlled(gt.type) ? gt.control : -1};
    for (int q : qs)
      if (q >= low && !inA[q]) add++;
    if (low + used + add > K) {
      close_block(g0, g);
      g0 = g;
      used = 0;
    }
    for (int q : qs)
      if (q >= low && !inA[q]) {
        inA[q] = 1;
        used++;
      }
  };
  if (cuts.empty()) {
    for (int g = 0; g < c->L; g++) take_gate(g);
  } else {
    std::vector<int> mark(n, 0);
    int s0 = 0;
    for (int e : cuts) {  // partition [s0, e)
      std::vector<int> fresh;
      for (int g = s0; g < e; g++) {
        const Gate& gt = c->h_gates[g];
        int qs[2] = {gt.target, gate_controlled(gt.type) ? gt.control : -1};
        for (int q : qs)
          if (q >= low && !mark[q]) {
            mark[q] = 1;
            fresh.push_back(q);
          }
      }
      int add = 0, own = (int)fresh.size();
      for (int q : fresh) {
        if (!inA[q]) add++;
        mark[q] = 0;
      }
      if (low + own > K) {  // the partition alone exceeds the chunk
        for (int g = s0; g < e; g++) take_gate(g);
      } else {
        if (low + used + add > K) {
          close_block(g0, s0);
          g0 = s0;
          used = 0;
          add = own;
        }
        for (int q : fresh) inA[q] = 1;
        used += add;
      }
      s0 = e;
    }
  }
  if (c->L > 0) close_block(g0, c->L);
  if (c->L == 0) return SQG_OK;
  cudaError_t e = cudaMalloc(&c->d_lgates, sizeof(Gate) * c->L);
  if (e == cudaSuccess) e = cudaMemcpy(c->d_lgates, lg.data(), sizeof(Gate) * c->L, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_hitab, sizeof(int) * hitab.size());
  if (e == cudaSuccess) e = cudaMemcpy(c->d_hitab, hitab.data(), sizeof(int) * hitab.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_inact, sizeof(int) * inact.size());
  if (e == cudaSuccess) e = cudaMemcpy(c->d_inact, inact.data(), sizeof(int) * inact.size(), cudaMemcpyHostToDevice);
  return cuda_status(e, "state plan");
}

// One block of gates applied to every chunk of 2^K amplitudes of a state vector.  The
// chunk's low local bits are the state's lowest qubits (a warp loads 32 consecutive
// amplitudes), its high local bits are the block's other qubits (offsets from hitab), and the
// remaining qubits number the chunks (inact).  One read and one write of the state per block.
struct StateArgs {
  double2* states;
  long long stride;
  int n, K, low, g0, g1, L;
  const Gate* lgates;
  const GateMat* gm;
  const int* hitab;
  const int* inact;
};

__global__ void __launch_bounds__(kStateThreads) k_state_block(StateArgs a) {
  extern __shared__ double2 sv[];
  __shared__ int hit[128];
  const int b = blockIdx.y;
  const int KK = 1 << a.K, hb = a.K - a.low, lowmask = (1 << a.low) - 1;
  for (int h = threadIdx.x; h < (1 << hb); h += blockDim.x) hit[h] = a.hitab[h];
  long long cbase = 0;
  for (int j = 0; j < a.n - a.K; j++)
    if ((blockIdx.x >> j) & 1u) cbase |= 1LL << a.inact[j];
  double2* base = a.states + (long long)b * a.stride + cbase;
  __syncthreads();
  for (int l = threadIdx.x; l < KK; l += blockDim.x) sv[l] = base[(l & lowmask) + hit[l >> a.low]];
  __syncthreads();
  const GateMat* gmb = a.gm + (long long)b * a.L;
  for (int g = a.g0; g < a.g1; g++) {
    const Gate gt = a.lgates[g];
    tile_apply(sv, KK, a.K, 1, gt, make_op(gt.type, gmb[g], ORIENT_FWD));
    __syncthreads();
  }
  for (int l = threadIdx.x; l < KK; l += blockDim.x) base[(l & lowmask) + hit[l >> a.low]] = sv[l];
}

}  // namespace

// =====================================================================================
// C ABI
// =====================================================================================
// Merged forward plan: walking the gates in order, single-qubit gates collect per qubit; a
// two-qubit gate first emits the open runs of its two qubits, then itself; the remaining runs
// are emitted at the end.  This only moves single-qubit gates past gates on other qubits, with
// which they commute.  A run becomes one general 2x2 gate (16 FP64 instructions per amplitude
// pair) when its members cost more (U3 14, RX/RY/RZ 8), otherwise its members stay.  The plan is
// kept only if it removes work; the adjoint and right-application paths use the gates as given.
int build_merge_plan(sqg_circuit* c) {
  const std::vector<Gate>& g = c->h_gates;
  std::vector<std::vector<int>> open(c->n);
  std::vector<Gate> mg;
  std::vector<int> first{0}, members;
  bool merged = false;
  auto cost1 = [](int type) { return type == G_U3 ? 14 : 8; };
  auto emit_one = [&](int i) {
    mg.push_back(g[i]);
    members.push_back(i);
    first.push_back((int)members.size());
  };
  auto flush = [&](int q) {
    std::vector<int>& run = open[q];
    int sum = 0;
    for (int i : run) sum += cost1(g[i].type);
    if (run.size() >= 2 && sum > 16) {
      mg.push_back(Gate{G_GEN, q, -1, -1});
      members.insert(members.end(), run.begin(), run.end());
      first.push_back((int)members.size());
      merged = true;
    } else {
      for (int i : run) emit_one(i);
    }
    run.clear();
  };
  for (int i = 0; i < c->L; i++) {
    if (gate_controlled(g[i].type)) {
      flush(g[i].target);
      flush(g[i].control);
      emit_one(i);
    } else {
      open[g[i].target].push_back(i);
    }
  }
  for (int q = 0; q < c->n; q++) flush(q);
  if (!merged) return SQG_OK;
  c->Lm = (int)mg.size();
  cudaError_t e = cudaMalloc(&c->d_mgates, sizeof(Gate) * mg.size());
  if (e == cudaSuccess) e = cudaMalloc(&c->d_mfirst, sizeof(int) * first.size());
  if (e == cudaSuccess) e = cudaMalloc(&c->d_mmembers, sizeof(int) * members.size());
  if (e == cudaSuccess) e = cudaMemcpy(c->d_mgates, mg.data(), sizeof(Gate) * mg.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(c->d_mfirst, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(c->d_mmembers, members.data(), sizeof(int) * members.size(), cudaMemcpyHostToDevice);
  return cuda_status(e, "merged forward plan");
}

extern "C" {

const char* sqg_status_string(int status) {
  switch (status) {
    case SQG_OK: return "ok";
    case SQG_ERR_INVALID_ARGUMENT: return "invalid argument";
    case SQG_ERR_UNSUPPORTED: return "unsupported configuration";
    case SQG_ERR_WORKSPACE: return "workspace too small";
    case SQG_ERR_CUDA: return "CUDA error";
    case SQG_ERR_PARAMETER_COUNT: return "wrong number of parameters";
    default: return "unknown status";
  }
}

const char* sqg_last_error(void) { return g_last_error.c_str(); }

int sqg_circuit_create(int qbit_num, const sqg_gate* gates, int gate_num, sqg_circuit** out) {
  if (!out) return fail(SQG_ERR_INVALID_ARGUMENT, "null output handle");
  *out = nullptr;
  if (qbit_num < 1 || qbit_num > kStateQubits) return fail(SQG_ERR_UNSUPPORTED, "qbit_num must be in 1..30");
  if (gate_num < 0 || (gate_num > 0 && !gates)) return fail(SQG_ERR_INVALID_ARGUMENT, "bad gate list");
  auto* c = new sqg_circuit();
  c->n = qbit_num;
  c->N = 1 << qbit_num;
  c->L = gate_num;
  int p = 0;
  for (int i = 0; i < gate_num; i++) {
    const sqg_gate& g = gates[i];
    int t = g.type;
    bool known = t == G_CZ || t == G_CNOT || t == G_U3 || t == G_RY || t == G_RX || t == G_RZ || t == G_CRY;
    if (!known) {
      delete c;
      return fail(SQG_ERR_UNSUPPORTED, "gate " + std::to_string(i) + ": unsupported gate type " + std::to_string(t));
    }
    if (g.target < 0 || g.target >= qbit_num) {
      delete c;
      return fail(SQG_ERR_INVALID_ARGUMENT, "gate " + std::to_string(i) + ": target qubit out of range");
    }
    if (gate_controlled(t) && (g.control < 0 || g.control >= qbit_num || g.control == g.target)) {
      delete c;
      return fail(SQG_ERR_INVALID_ARGUMENT, "gate " + std::to_string(i) + ": bad control qubit");
    }
    if (g.param_start != p) {
      delete c;
      return fail(SQG_ERR_INVALID_ARGUMENT, "gate " + std::to_string(i) + ": parameters must be contiguous in gate order");
    }
    if (gate_controlled(t) && qbit_num < 2) {
      delete c;
      return fail(SQG_ERR_INVALID_ARGUMENT, "controlled gate needs two qubits");
    }
    Gate d{t, g.target, gate_controlled(t) ? g.control : -1, g.param_start};
    c->h_gates.push_back(d);
    p += gate_param_num(t);
  }
  c->P = p;
  cudaGetDevice(&c->device);
  if (gate_num > 0) {
    cudaError_t e = cudaMalloc(&c->d_gates, sizeof(Gate) * gate_num);
    if (e == cudaSuccess) e = cudaMemcpy(c->d_gates, c->h_gates.data(), sizeof(Gate) * gate_num, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      int st = cuda_status(e, "sqg_circuit_create");
      sqg_circuit_destroy(c);
      return st;
    }
  }
  int st = build_state_plan(c);
  if (!st) st = build_merge_plan(c);
  if (st) {
    sqg_circuit_destroy(c);
    return st;
  }
  *out = c;
  return SQG_OK;
}

int sqg_circuit_set_partitions(sqg_circuit* c, const int* part_ends, int nparts) {
  if (!c) return fail(SQG_ERR_INVALID_ARGUMENT, "null circuit handle");
  if (nparts < 0 || (nparts > 0 && !part_ends)) return fail(SQG_ERR_INVALID_ARGUMENT, "bad partition list");
  std::vector<int> cuts(part_ends, part_ends + nparts);
  for (int i = 0; i < nparts; i++)
    if (cuts[i] < (i ? cuts[i - 1] : 0) || cuts[i] > c->L)
      return fail(SQG_ERR_INVALID_ARGUMENT, "partition ends must be non-decreasing gate indices <= gate_num");
  if (nparts > 0 && cuts.back() != c->L) return fail(SQG_ERR_INVALID_ARGUMENT, "the last partition must end at gate_num");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != c->device) return fail(SQG_ERR_INVALID_ARGUMENT, "circuit handle belongs to another device");
  cudaFree(c->d_lgates);
  cudaFree(c->d_hitab);
  cudaFree(c->d_inact);
  c->d_lgates = nullptr;
  c->d_hitab = nullptr;
  c->d_inact = nullptr;
  c->sblocks.clear();
  return build_state_plan(c, cuts);
}

int sqg_circuit_destroy(sqg_circuit* c) {
  if (!c) return SQG_OK;
  if (c->d_gates) cudaFree(c->d_gates);
  if (c->d_lgates) cudaFree(c->d_lgates);
  if (c->d_hitab) cudaFree(c->d_hitab);
  if (c->d_inact) cudaFree(c->d_inact);
  if (c->d_mgates) cudaFree(c->d_mgates);
  if (c->d_mfirst) cudaFree(c->d_mfirst);
  if (c->d_mmembers) cudaFree(c->d_mmembers);
  delete c;
  return SQG_OK;
}

int sqg_circuit_param_num(const sqg_circuit* c) { return c ? c->P : -1; }
int sqg_circuit_qbit_num(const sqg_circuit* c) { return c ? c->n : -1; }
int sqg_circuit_gate_num(const sqg_circuit* c) { return c ? c->L : -1; }

size_t sqg_cost_grad_workspace_bytes(const sqg_circuit* c, int batch, int cols, int with_grad) {
  if (!c || batch <= 0 || cols <= 0) return 0;
  return eval_layout(c, batch, cols, with_grad != 0, 0).end;
}

size_t sqg_cost_grad_checkpoint_workspace_bytes(const sqg_circuit* c, int batch, int cols, int checkpoint_interval) {
  if (!c || batch <= 0 || cols <= 0) return 0;
  return eval_layout(c, batch, cols, true, checkpoint_interval).end;
}

// Argument checks of sqg_cost_grad, shared with sqg_cost_grad_noalloc.
static int cost_grad_args(const sqg_circuit* c, const double* theta, int B, const void* target, int cols,
                          int trace_offset, int variant, const double* cost, const double* grad,
                          int checkpoint_interval) {
  int st = check_circuit(c);
  if (st) return st;
  if (B <= 0 || B > 65535 || !target || !cost || cols <= 0)
    return fail(SQG_ERR_INVALID_ARGUMENT, "bad batch (1..65535), target or output");
  if (c->P > 0 && !theta) return fail(SQG_ERR_INVALID_ARGUMENT, "null parameter array");
  if (cols > c->N) return fail(SQG_ERR_INVALID_ARGUMENT, "target has more columns than rows");
  if (variant != SQG_FROBENIUS_NORM && variant != SQG_HILBERT_SCHMIDT_TEST && variant != SQG_INFIDELITY)
    return fail(SQG_ERR_UNSUPPORTED, "cost function variant not implemented by the engine");
  const int off = variant == SQG_FROBENIUS_NORM ? trace_offset : 0;
  if (off < 0 || off + cols > c->N) return fail(SQG_ERR_INVALID_ARGUMENT, "trace offset out of range");
  const bool with_grad = grad != nullptr && c->P > 0;
  if (with_grad && c->n > 12) return fail(SQG_ERR_UNSUPPORTED, "gradient supports qbit_num <= 12");
  if (checkpoint_interval < 0) return fail(SQG_ERR_INVALID_ARGUMENT, "negative checkpoint interval");
  return SQG_OK;
}

int sqg_cost_grad(const sqg_circuit* c, const double* theta, int B, const void* target, int cols,
                  long long target_batch_stride, int trace_offset, int variant, double* cost, double* grad,
                  int checkpoint_interval, void* workspace, size_t ws_bytes, void* stream) {
  int st = cost_grad_args(c, theta, B, target, cols, trace_offset, variant, cost, grad, checkpoint_interval);
  if (st) return st;
  const int off = variant == SQG_FROBENIUS_NORM ? trace_offset : 0;
  const bool with_grad = grad != nullptr && c->P > 0;
  if (with_grad && checkpoint_interval == 0) {
    // up to five qubits: one CTA per vector with the environment-matrix evaluation
    st = sqg::env_cost_grad(c, theta, B, target, cols, target_batch_stride, off, variant, cost, grad, stream);
    if (st != SQG_ERR_UNSUPPORTED) return st;
    st = SQG_OK;
  }
  EvalLayout l = eval_layout(c, B, cols, with_grad, with_grad ? checkpoint_interval : 0);
  if (!workspace || ws_bytes < l.end) return fail(SQG_ERR_WORKSPACE, "workspace too small: need " + std::to_string(l.end));
  cudaStream_t s = (cudaStream_t)stream;
  char* ws = (char*)workspace;
  GateMat* gm = (GateMat*)(ws + l.prep.gm_off);
  double2* sc = (double2*)(ws + l.prep.sc_off);
  double2* wtr = (double2*)(ws + l.tr_off);
  double2* wgr = (double2*)(ws + l.gr_off);
  if ((st = launch_prep(c, theta, c->P, B, gm, sc, s))) return st;
  TileArgs a;
  a.gates = c->d_gates;
  a.L = c->L; a.P = c->P; a.n = c->n; a.N = c->N;
  a.gm = gm; a.sc = sc;
  a.mtx = (double2*)target;
  a.bstride = target_batch_stride;
  a.rstride = cols;
  a.cstride = 1;
  a.cols = cols;
  a.TC = l.plan.TC;
  a.tiles = l.plan.tiles;
  a.trace_offset = off;
  a.reverse_order = 0;
  a.orient = ORIENT_FWD;
  a.ws_tr = wtr;
  a.ws_gr = wgr;
  a.ckpt = l.nck > 0 ? (double2*)(ws + l.ck_off) : nullptr;
  a.ckpt_interval = checkpoint_interval;
  a.nck = l.nck;
  dim3 grid(l.plan.tiles, B);
  if (with_grad) {
    if ((st = set_smem(k_tile_adjoint, l.plan.smem))) return st;
    k_tile_adjoint<<<grid, l.plan.threads, l.plan.smem, s>>>(a);
  } else {
    if ((st = forward_plan(c, l.prep, ws, B, gm, a, s))) return st;
    if ((st = set_smem(k_tile_forward<false, true>, l.plan.smem))) return st;
    k_tile_forward<false, true><<<grid, l.plan.threads, l.plan.smem, s>>>(a);
  }
  if ((st = cuda_status(cudaGetLastError(), "tile kernel"))) return st;
  dim3 fgrid(B, with_grad ? (c->P + 127) / 128 : 1);
  k_finish<<<fgrid, 128, 0, s>>>(wtr, wgr, l.plan.tiles, c->P, cols, variant, cost, with_grad ? grad : nullptr);
  return cuda_status(cudaGetLastError(), "k_finish");
}

}  // extern "C"

// ---- allocation-free cost/gradient ---------------------------------------------------
// The scratch of sqg_cost_grad_noalloc: a file-scope device array of fixed size.  In host
// code its name is a host-side stand-in, not a device address; the device address is looked
// up with cudaGetSymbolAddress in the CUDA context that is current for the call, once per
// context (a device normally has one, its primary context; a cudaDeviceReset or a driver-API
// context made current gives the device another, and the array another address).
static __device__ __align__(256) unsigned char g_noalloc_scratch[SQG_NOALLOC_SCRATCH_BYTES];

namespace {
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

struct NoallocSlot {
  unsigned long long ctx_id;
  void* addr;
};
constexpr int kNoallocSlots = 64;
std::mutex g_noalloc_mu;
NoallocSlot g_noalloc_slots[kNoallocSlots] = {};
int g_noalloc_used = 0;
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;

// Unique id of the current CUDA context (*have = false when none is current).  The two
// driver functions are reached through the runtime's entry-point lookup, so the library
// does not link the driver library itself.
int current_context(unsigned long long* id, bool* have) {
  if (!g_ctx_current || !g_ctx_id) {
    cudaDriverEntryPointQueryResult q1, q2;
    cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", (void**)&g_ctx_current, 12000,
                                                      cudaEnableDefault, &q1);
    cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", (void**)&g_ctx_id, 12000, cudaEnableDefault, &q2);
    if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
        q2 != cudaDriverEntryPointSuccess || !g_ctx_current || !g_ctx_id) {
      g_ctx_current = nullptr;
      g_ctx_id = nullptr;
      return fail(SQG_ERR_CUDA, "cannot reach cuCtxGetCurrent/cuCtxGetId through the CUDA runtime");
    }
  }
  CUcontext ctx = nullptr;
  if (g_ctx_current(&ctx) != CUDA_SUCCESS) return fail(SQG_ERR_CUDA, "cuCtxGetCurrent failed");
  *have = ctx != nullptr;
  if (!ctx) return SQG_OK;
  if (g_ctx_id(ctx, id) != CUDA_SUCCESS) return fail(SQG_ERR_CUDA, "cuCtxGetId failed");
  return SQG_OK;
}

// Device address of the scratch array in the current context.
int noalloc_scratch(void** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  unsigned long long id = 0;
  bool have = false;
  int st = current_context(&id, &have);
  if (st) return st;
  if (have) {
    for (int i = 0; i < g_noalloc_used && i < kNoallocSlots; ++i)
      if (g_noalloc_slots[i].ctx_id == id) {
        *out = g_noalloc_slots[i].addr;
        return SQG_OK;
      }
  }
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(no-alloc scratch)");
  if (!have) {  // the runtime has just made its context current
    if ((st = current_context(&id, &have))) return st;
    if (!have) return fail(SQG_ERR_CUDA, "no CUDA context is current after cudaGetSymbolAddress");
  }
  g_noalloc_slots[g_noalloc_used % kNoallocSlots] = {id, p};
  ++g_noalloc_used;
  *out = p;
  return SQG_OK;
}
}  // namespace

extern "C" {

int sqg_cost_grad_noalloc(const sqg_circuit* c, const double* theta, int B, const void* target, int cols,
                          long long target_batch_stride, int trace_offset, int variant, double* cost, double* grad,
                          int checkpoint_interval, void* stream) {
  int st = cost_grad_args(c, theta, B, target, cols, trace_offset, variant, cost, grad, checkpoint_interval);
  if (st) return st;
  const bool with_grad = grad != nullptr && c->P > 0;
  if (with_grad && checkpoint_interval == 0) {
    // up to five qubits the environment-matrix form takes no scratch at all
    const int off = variant == SQG_FROBENIUS_NORM ? trace_offset : 0;
    st = sqg::env_cost_grad(c, theta, B, target, cols, target_batch_stride, off, variant, cost, grad, stream);
    if (st != SQG_ERR_UNSUPPORTED) return st;
  }
  const size_t need = eval_layout(c, B, cols, with_grad, with_grad ? checkpoint_interval : 0).end;
  if (need > SQG_NOALLOC_SCRATCH_BYTES)
    return fail(SQG_ERR_WORKSPACE, "sqg_cost_grad_noalloc: this call needs " + std::to_string(need) +
                                       " bytes of scratch but the built-in array holds " +
                                       std::to_string((size_t)SQG_NOALLOC_SCRATCH_BYTES) +
                                       "; use sqg_cost_grad with a caller-allocated workspace or a smaller batch");
  void* ws = nullptr;
  if ((st = noalloc_scratch(&ws))) return st;
  return sqg_cost_grad(c, theta, B, target, cols, target_batch_stride, trace_offset, variant, cost, grad,
                       checkpoint_interval, ws, SQG_NOALLOC_SCRATCH_BYTES, stream);
}

size_t sqg_apply_workspace_bytes(const sqg_circuit* c, int batch) {
  if (!c || batch <= 0) return 0;
  return prep_layout(c, batch, 0).end;
}

int sqg_apply(const sqg_circuit* c, const double* theta, int B, void* mtx, int cols, long long stride,
              long long batch_stride, int fused, void* workspace, size_t ws_bytes, void* stream) {
  int st = check_circuit(c);
  if (st) return st;
  if (B <= 0 || B > 65535 || !mtx || cols <= 0 || stride < cols)
    return fail(SQG_ERR_INVALID_ARGUMENT, "bad matrix arguments");
  if (c->P > 0 && !theta) return fail(SQG_ERR_INVALID_ARGUMENT, "null parameter array");
  PrepLayout l = prep_layout(c, B, 0);
  if (!workspace || ws_bytes < l.end) return fail(SQG_ERR_WORKSPACE, "workspace too small: need " + std::to_string(l.end));
  if (c->L == 0) return SQG_OK;
  cudaStream_t s = (cudaStream_t)stream;
  char* ws = (char*)workspace;
  GateMat* gm = (GateMat*)(ws + l.gm_off);
  double2* sc = (double2*)(ws + l.sc_off);
  if ((st = launch_prep(c, theta, c->P, B, gm, sc, s))) return st;
  if (fused) {
    TilePlan pl = plan_tiles(c->N, cols, false);
    TileArgs a;
    memset(&a, 0, sizeof(a));
    a.gates = c->d_gates;
    a.L = c->L; a.P = c->P; a.n = c->n; a.N = c->N;
    a.gm = gm; a.sc = sc;
    a.mtx = (double2*)mtx;
    a.bstride = batch_stride;
    a.rstride = stride;
    a.cstride = 1;
    a.cols = cols;
    a.TC = pl.TC;
    a.tiles = pl.tiles;
    a.orient = ORIENT_FWD;
    if ((st = forward_plan(c, l, ws, B, gm, a, s))) return st;
    if ((st = set_smem(k_tile_forward<true, false>, pl.smem))) return st;
    k_tile_forward<true, false><<<dim3(pl.tiles, B), pl.threads, pl.smem, s>>>(a);
    return cuda_status(cudaGetLastError(), "k_tile_forward");
  }
  // unfused: one pass over the matrix per gate
  for (int b = 0; b < B; b++) {
    double2* base = (double2*)mtx + (long long)b * batch_stride;
    for (int g = 0; g < c->L; g++) {
      const Gate& gt = c->h_gates[g];
      if ((gt.type == G_CNOT || gt.type == G_CZ) && c->n >= 2) {
        const int shift = (cols & (cols - 1)) == 0 ? __builtin_ctz((unsigned)cols) : -1;
        const long long items = (long long)cols << (c->n - 2);
        const int blocks = (int)std::min<long long>((items + 1023) / 1024, 152LL * 16);
        if (gt.type == G_CNOT)
          k_perm_hbm<0><<<blocks, 256, 0, s>>>(base, stride, cols, shift, items, gt.target, gt.control);
        else
          k_perm_hbm<1><<<blocks, 256, 0, s>>>(base, stride, cols, shift, items, gt.target, gt.control);
        continue;
      }
      long long items = (long long)cols << (gate_controlled(gt.type) ? c->n - 2 : c->n - 1);
      k_gate_hbm<<<dim3(hbm_blocks(items), 1), 256, 0, s>>>(base, 0, stride, cols, c->n, gt, gm + (long long)b * c->L + g,
                                                          sc + (long long)b * c->P, -1, 1);
    }
  }
  return cuda_status(cudaGetLastError(), "k_gate_hbm");
}

int sqg_apply_from_right(const sqg_circuit* c, const double* theta, void* mtx, int rows, long long stride,
                         void* workspace, size_t ws_bytes, void* stream) {
  int st = check_circuit(c);
  if (st) return st;
  if (!mtx || rows <= 0 || stride < c->N) return fail(SQG_ERR_INVALID_ARGUMENT, "bad matrix arguments");
  if (c->P > 0 && !theta) return fail(SQG_ERR_INVALID_ARGUMENT, "null parameter array");
  PrepLayout l = prep_layout(c, 1, 0);
  if (!workspace || ws_bytes < l.end) return fail(SQG_ERR_WORKSPACE, "workspace too small: need " + std::to_string(l.end));
  if (c->L == 0) return SQG_OK;
  cudaStream_t s = (cudaStream_t)stream;
  char* ws = (char*)workspace;
  GateMat* gm = (GateMat*)(ws + l.gm_off);
  double2* sc = (double2*)(ws + l.sc_off);
  if ((st = launch_prep(c, theta, c->P, 1, gm, sc, s))) return st;
  TilePlan pl = plan_tiles(c->N, rows, false);
  TileArgs a;
  memset(&a, 0, sizeof(a));
  a.gates = c->d_gates;
  a.L = c->L; a.P = c->P; a.n = c->n; a.N = c->N;
  a.gm = gm; a.sc = sc;
  a.mtx = (double2*)mtx;
  a.bstride = 0;
  a.rstride = stride;
  a.cstride = 0;  // vectors are rows
  a.cols = rows;
  a.TC = pl.TC;
  a.tiles = pl.tiles;
  a.reverse_order = 1;
  a.orient = ORIENT_TRANS;
  if ((st = set_smem(k_tile_forward<true, false>, pl.smem))) return st;
  k_tile_forward<true, false><<<dim3(pl.tiles, 1), pl.threads, pl.smem, s>>>(a);
  return cuda_status(cudaGetLastError(), "k_tile_forward(right)");
}

int sqg_combined_unitary(const sqg_circuit* c, const double* theta, const void* target, int cols, void* out,
                         void* workspace, size_t ws_bytes, void* stream) {
  int st = check_circuit(c);
  if (st) return st;
  if (!target || !out || cols <= 0) return fail(SQG_ERR_INVALID_ARGUMENT, "bad matrix arguments");
  if (c->P > 0 && !theta) return fail(SQG_ERR_INVALID_ARGUMENT, "null parameter array");
  PrepLayout l = prep_layout(c, 1, 0);
  if (!workspace || ws_bytes < l.end) return fail(SQG_ERR_WORKSPACE, "workspace too small: need " + std::to_string(l.end));
  cudaStream_t s = (cudaStream_t)stream;
  char* ws = (char*)workspace;
  GateMat* gm = (GateMat*)(ws + l.gm_off);
  double2* sc = (double2*)(ws + l.sc_off);
  const long long msz = (long long)c->N * cols;
  double2* o = (double2*)out;
  cudaError_t e = cudaMemcpyAsync(o, target, sizeof(double2) * msz, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_status(e, "sqg_combined_unitary");
  if (c->L == 0) return SQG_OK;
  if ((st = launch_prep(c, theta, c->P, 1, gm, sc, s))) return st;
  // out[0] carries the forward state; derivative outputs out[1+k] are created from the
  // state in front of their gate and then carried through the remaining gates
  // (Gates_block::apply_derivate_to, Gates_block.cpp:1012-1150).
  int created = 0;
  for (int g = 0; g < c->L; g++) {
    const Gate& gt = c->h_gates[g];
    int np = gate_param_num(gt.type);
    for (int k = 0; k < np; k++) {
      double2* d = o + msz * (1 + gt.pstart + k);
      e = cudaMemcpyAsync(d, o, sizeof(double2) * msz, cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return cuda_status(e, "sqg_combined_unitary");
      long long items = (long long)cols << (c->n - 1);
      k_gate_hbm<<<dim3(hbm_blocks(items), 1), 256, 0, s>>>(d, 0, cols, cols, c->n, gt, gm + g, sc, k, 1);
    }
    // forward gate on out[0] and on the derivative outputs created before this gate
    int nmat = 1 + created;
    long long items = (long long)cols << (gate_controlled(gt.type) ? c->n - 2 : c->n - 1);
    k_gate_hbm<<<dim3(hbm_blocks(items), std::min(nmat, 65535)), 256, 0, s>>>(o, msz, cols, cols, c->n, gt, gm + g, sc,
                                                                             -1, nmat);
    created += np;
  }
  return cuda_status(cudaGetLastError(), "sqg_combined_unitary");
}


size_t sqg_state_workspace_bytes(const sqg_circuit* c, int batch) {
  if (!c || batch <= 0) return 0;
  return prep_layout(c, batch, 0).end;
}

int sqg_state_block_count(const sqg_circuit* c) { return c ? (int)c->sblocks.size() : -1; }

int sqg_apply_state(const sqg_circuit* c, const double* theta, int B, void* states, long long stride, int fused,
                    void* workspace, size_t ws_bytes, void* stream) {
  int st = check_circuit(c, kStateQubits);
  if (st) return st;
  if (B <= 0 || B > 65535 || !states || stride < (long long)c->N)
    return fail(SQG_ERR_INVALID_ARGUMENT, "bad state arguments (batch 1..65535, stride >= 2^qbit_num)");
  if (c->P > 0 && !theta) return fail(SQG_ERR_INVALID_ARGUMENT, "null parameter array");
  PrepLayout l = prep_layout(c, B, 0);
  if (!workspace || ws_bytes < l.end) return fail(SQG_ERR_WORKSPACE, "workspace too small: need " + std::to_string(l.end));
  if (c->L == 0) return SQG_OK;
  cudaStream_t s = (cudaStream_t)stream;
  char* ws = (char*)workspace;
  GateMat* gm = (GateMat*)(ws + l.gm_off);
  double2* sc = (double2*)(ws + l.sc_off);
  if ((st = launch_prep(c, theta, c->P, B, gm, sc, s))) return st;
  if (fused) {
    const size_t smem = sizeof(double2) << c->sK;
    if ((st = set_smem(k_state_block, smem))) return st;
    StateArgs a;
    a.states = (double2*)states;
    a.stride = stride;
    a.n = c->n;
    a.K = c->sK;
    a.low = std::min(c->sK, kStateLow);
    a.L = c->L;
    a.lgates = c->d_lgates;
    a.gm = gm;
    for (size_t k = 0; k < c->sblocks.size(); k++) {
      a.g0 = c->sblocks[k].g0;
      a.g1 = c->sblocks[k].g1;
      a.hitab = c->d_hitab + 128 * k;
      a.inact = c->d_inact + 32 * k;
      k_state_block<<<dim3(1u << (c->n - c->sK), B), kStateThreads, smem, s>>>(a);
    }
    return cuda_status(cudaGetLastError(), "k_state_block");
  }
  // unfused: one pass over the state per gate
  for (int b = 0; b < B; b++) {
    double2* base = (double2*)states + (long long)b * stride;
    for (int g = 0; g < c->L; g++) {
      const Gate& gt = c->h_gates[g];
      long long items = 1LL << (gate_controlled(gt.type) ? c->n - 2 : c->n - 1);
      k_gate_hbm<<<dim3(hbm_blocks(items), 1), 256, 0, s>>>(base, 0, 1, 1, c->n, gt, gm + (long long)b * c->L + g,
                                                          sc + (long long)b * c->P, -1, 1);
    }
  }
  return cuda_status(cudaGetLastError(), "k_gate_hbm");
}

}  // extern "C"
