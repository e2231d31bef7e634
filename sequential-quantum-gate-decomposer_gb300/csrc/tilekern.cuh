// Column-tile kernel bodies shared by the fixed-shape launches (engine.cu) and the
// persistent ragged-batch launch (ragged.cu).  Each body processes one (instance, tile)
// work item with all threads of the CTA; smem holds the tile(s) plus reduction scratch.
#pragma once
#include "gates.cuh"
#include "tile.cuh"

namespace sqg {

struct TileArgs {
  const Gate* gates;
  int L, P, n, N;
  const GateMat* gm;   // [B][L]
  const double2* sc;   // [B][P]
  // matrix source (target or in/out matrix); element (r, c) of instance b at
  // base + b*bstride + r*rstride + c*cstride
  double2* mtx;
  long long bstride, rstride, cstride;
  int cols;          // number of vectors (columns for left application, rows for right)
  int TC;            // vectors per tile
  int tiles;         // tiles per instance
  int trace_offset;  // row offset of the traced element (left application)
  int reverse_order; // right application walks the gates from last to first
  int orient;        // ORIENT_FWD or ORIENT_TRANS
  double2* ws_tr;    // [B][tiles] forward trace partials
  double2* ws_gr;    // [B][tiles][P] derivative trace partials
  double2* ckpt;     // checkpoints [B][tiles][nck][TC][N] or null
  int ckpt_interval;
  int nck;
};

__device__ __forceinline__ void load_tile(double2* s, const TileArgs& a, int b, int v0, int tc) {
  const double2* base = a.mtx + (long long)b * a.bstride;
  const int total = a.N * tc;
  if (a.cstride == 1) {
    // left application: vector = column, element r at row r; read rows coalesced
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
      int r = e / tc, c = e - r * tc;
      s[c * a.N + r] = base[(long long)r * a.rstride + v0 + c];
    }
  } else {
    // right application: vector = row (contiguous)
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
      int c = e / a.N, r = e - c * a.N;
      s[c * a.N + r] = base[(long long)(v0 + c) * a.rstride + r];
    }
  }
}

__device__ __forceinline__ void store_tile(const double2* s, const TileArgs& a, int b, int v0, int tc) {
  double2* base = a.mtx + (long long)b * a.bstride;
  const int total = a.N * tc;
  if (a.cstride == 1) {
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
      int r = e / tc, c = e - r * tc;
      base[(long long)r * a.rstride + v0 + c] = s[c * a.N + r];
    }
  } else {
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
      int c = e / a.N, r = e - c * a.N;
      base[(long long)(v0 + c) * a.rstride + r] = s[c * a.N + r];
    }
  }
}

// Gate records and 2x2 matrices are staged in shared memory kGateChunk at a time, so each
// CTA reads them from global memory once instead of once per warp and gate.
constexpr int kGateChunk = kStage;
constexpr size_t kGateStageBytes = kGateChunk * (sizeof(Gate) + sizeof(GateMat));

// Forward (or right) application of the whole circuit to one tile; optionally writes
// the tile back and/or the traced diagonal partial.
template <bool WRITE_BACK, bool TRACE>
__device__ __forceinline__ void tile_forward_body(const TileArgs& a, int b, int tile, double2* smem) {
  double2* s = smem;
  double2* red = smem + (size_t)a.TC * a.N;
  GateMat* gst = reinterpret_cast<GateMat*>(red + kTileMaxWarps);  // [kGateChunk]
  Gate* gts = reinterpret_cast<Gate*>(gst + kGateChunk);            // [kGateChunk]
  const int v0 = tile * a.TC;
  const int tc = min(a.TC, a.cols - v0);
  const int logN = a.n;
  load_tile(s, a, b, v0, tc);
  const GateMat* gm = a.gm + (long long)b * a.L;
  for (int k0 = 0; k0 < a.L; k0 += kGateChunk) {
    const int kn = min(kGateChunk, a.L - k0);
    __syncthreads();  // the previous chunk's records are no longer read
    if (threadIdx.x < kn) {
      const int k = k0 + threadIdx.x;
      const int g = a.reverse_order ? a.L - 1 - k : k;
      gts[threadIdx.x] = a.gates[g];
      gst[threadIdx.x] = gm[g];
    }
    __syncthreads();
    for (int j = 0; j < kn; j++) {
      const Gate gt = gts[j];
      PairOp op = make_op(gt.type, gst[j], a.orient);
      tile_apply(s, a.N, logN, tc, gt, op);
      __syncthreads();
    }
  }
  __syncthreads();
  if (TRACE) {
    double2 t = tile_trace(s, a.N, tc, v0, a.trace_offset, reinterpret_cast<double*>(red));
    if (threadIdx.x == 0) a.ws_tr[(long long)b * a.tiles + tile] = t;
  }
  if (WRITE_BACK) store_tile(s, a, b, v0, tc);
}

// Cost + adjoint gradient of one (instance, tile).
__device__ __forceinline__ void tile_adjoint_body(const TileArgs& a, int b, int tile, double2* smem) {
  const int N = a.N, logN = a.n;
  double2* psi = smem;
  double2* lam = smem + (size_t)a.TC * N;
  double* redd = reinterpret_cast<double*>(lam + (size_t)a.TC * N);  // [kTileMaxWarps][8]
  double* tot = redd + kTileMaxWarps * 8;                             // [8]
  double* scratch = tot + 8;                                          // [kTileMaxWarps]
  GateMat* gst = reinterpret_cast<GateMat*>(scratch + kTileMaxWarps);  // [kGateChunk]
  Gate* gts = reinterpret_cast<Gate*>(gst + kGateChunk);              // [kGateChunk]
  const int v0 = tile * a.TC;
  const int tc = min(a.TC, a.cols - v0);
  const size_t tile_elems = (size_t)a.TC * N;
  double2* ck = a.ckpt ? a.ckpt + ((long long)b * a.tiles + tile) * a.nck * tile_elems : nullptr;

  load_tile(psi, a, b, v0, tc);
  // lambda_j = e_{j + offset}
  for (int e = threadIdx.x; e < tc * N; e += blockDim.x) {
    int c = e / N, r = e - c * N;
    lam[e] = make_double2(r == v0 + c + a.trace_offset ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
  const GateMat* gm = a.gm + (long long)b * a.L;
  const double2* scb = a.sc + (long long)b * a.P;
  // forward sweep, storing psi after every ckpt_interval-th gate
  for (int g = 0; g < a.L; g++) {
    const int j = g % kGateChunk;
    if (j == 0) {
      __syncthreads();
      if ((int)threadIdx.x < min(kGateChunk, a.L - g)) {
        gts[threadIdx.x] = a.gates[g + threadIdx.x];
        gst[threadIdx.x] = gm[g + threadIdx.x];
      }
      __syncthreads();
    }
    Gate gt = gts[j];
    PairOp op = make_op(gt.type, gst[j], ORIENT_FWD);
    tile_apply(psi, N, logN, tc, gt, op);
    __syncthreads();
    if (ck && (g + 1) % a.ckpt_interval == 0 && (g + 1) / a.ckpt_interval <= a.nck) {
      double2* dst = ck + (size_t)((g + 1) / a.ckpt_interval - 1) * tile_elems;
      for (int e = threadIdx.x; e < tc * N; e += blockDim.x) dst[e] = psi[e];
    }
  }
  double2 t = tile_trace(psi, N, tc, v0, a.trace_offset, scratch);
  if (threadIdx.x == 0) a.ws_tr[(long long)b * a.tiles + tile] = t;
  double2* wgr = a.ws_gr + ((long long)b * a.tiles + tile) * a.P;
  auto sink = [&](int, const Gate& gt, const double* R) {
    if (threadIdx.x < gate_param_num(gt.type)) wgr[gt.pstart + threadIdx.x] = contract_derivative(gt, scb, threadIdx.x, R);
  };
  // before reverse step g, psi must hold the state after gate g; restore the stored copy
  // at checkpoint boundaries so that uncomputation error never spans more than
  // ckpt_interval gates
  auto restore = [&](int g) {
    if (ck && (g + 1) % a.ckpt_interval == 0 && (g + 1) / a.ckpt_interval <= a.nck && g + 1 < a.L) {
      const double2* src = ck + (size_t)((g + 1) / a.ckpt_interval - 1) * tile_elems;
      __syncthreads();
      for (int e = threadIdx.x; e < tc * N; e += blockDim.x) psi[e] = src[e];
      __syncthreads();
    }
  };
  adjoint_sweep(psi, lam, N, logN, tc, a.gates, gm, scb, a.L, redd, tot, sink, restore, gts, gst);
}


// Shared memory bytes of one work item: tiles plus reduction scratch.
__host__ __device__ inline size_t tile_smem_bytes(int TC, int N, bool grad) {
  size_t per = (size_t)N * sizeof(double2) * (grad ? 2 : 1);
  size_t extra = grad ? (kTileMaxWarps * 8 + 8 + kTileMaxWarps) * sizeof(double) + kGateStageBytes
                      : kTileMaxWarps * sizeof(double2) + kGateStageBytes;
  return per * TC + extra;
}

}  // namespace sqg
