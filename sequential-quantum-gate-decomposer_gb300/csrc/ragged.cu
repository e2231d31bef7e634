// Ragged batches: one launch evaluates instances that each have their own circuit (and so
// their own qubit count, gate list and parameter count) and their own target.  A
// persistent grid (CTAs resident on every SM) pulls (instance, tile) work items from a
// queue ordered by decreasing work, so large instances start first and small ones fill
// the tail.  Tile bodies are the ones of the fixed-shape launches (tilekern.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/sqg.h"
#include "gates.cuh"
#include "handle.h"
#include "tile.cuh"
#include "tilekern.cuh"

using namespace sqg;

namespace {

constexpr int kRaggedThreads = 256;

struct InstDesc {
  const Gate* gates;
  int L, P, n, N, cols, TC, tiles;
  long long theta_off, target_off, gm_off, sc_off, tr_off, gr_off;
};

}  // namespace

struct sqg_ragged_batch {
  int count = 0, with_grad = 0, device = 0, grid = 0, n_items = 0;
  size_t smem = 0;
  InstDesc* d_desc = nullptr;
  int2* d_items = nullptr;     // (instance, tile), decreasing work
  int2* d_gate_map = nullptr;  // (instance, gate) for every gate of the batch
  int total_gates = 0, maxP = 1;
  long long total_gm = 0, total_sc = 0, total_tr = 0, total_gr = 0;
  std::vector<long long> theta_off, target_off;
  size_t off_gm = 0, off_sc = 0, off_tr = 0, off_gr = 0, ws_bytes = 0;
};

namespace {

inline size_t a256(size_t v) { return (v + 255) / 256 * 256; }

__global__ void k_ragged_prep(const InstDesc* __restrict__ desc, const int2* __restrict__ gate_map, int total_gates,
                              const double* __restrict__ theta, GateMat* __restrict__ gm, double2* __restrict__ sc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total_gates) return;
  int2 m = gate_map[i];
  const InstDesc d = desc[m.x];
  const Gate gt = d.gates[m.y];
  const double* th = theta + d.theta_off + gt.pstart;
  double2* scb = sc + d.sc_off + gt.pstart;
  GateMat g;
  g.u[0] = g.u[1] = g.u[2] = g.u[3] = make_double2(0.0, 0.0);
  if (gt.type == G_U3) {
    double st, ct, sp, cp, sl, cl;
    sincos(th[0], &st, &ct);
    sincos(th[1], &sp, &cp);
    sincos(th[2], &sl, &cl);
    scb[0] = make_double2(st, ct);
    scb[1] = make_double2(sp, cp);
    scb[2] = make_double2(sl, cl);
    double spl = sp * cl + cp * sl, cpl = cp * cl - sp * sl;
    g.u[0] = make_double2(ct, 0.0);
    g.u[1] = make_double2(-st * cl, -st * sl);
    g.u[2] = make_double2(st * cp, st * sp);
    g.u[3] = make_double2(ct * cpl, ct * spl);
  } else if (gate_param_num(gt.type) == 1) {
    double s, c;
    sincos(th[0], &s, &c);
    scb[0] = make_double2(s, c);
    g.u[0] = make_double2(c, s);
  }
  gm[d.gm_off + m.y] = g;
}

template <bool GRAD>
__global__ void __launch_bounds__(kRaggedThreads) k_ragged_tiles(const InstDesc* __restrict__ desc,
                                                                 const int2* __restrict__ items, int n_items,
                                                                 int* __restrict__ counter, const double2* targets,
                                                                 const GateMat* gm, const double2* sc, double2* ws_tr,
                                                                 double2* ws_gr) {
  extern __shared__ double2 smem[];
  __shared__ int item_s;
  for (;;) {
    if (threadIdx.x == 0) item_s = atomicAdd(counter, 1);
    __syncthreads();
    const int item = item_s;
    __syncthreads();
    if (item >= n_items) break;
    const int2 it = items[item];
    const InstDesc d = desc[it.x];
    TileArgs a;
    a.gates = d.gates;
    a.L = d.L; a.P = d.P; a.n = d.n; a.N = d.N;
    a.gm = gm + d.gm_off;
    a.sc = sc + d.sc_off;
    a.mtx = const_cast<double2*>(targets) + d.target_off;
    a.bstride = 0;
    a.rstride = d.cols;
    a.cstride = 1;
    a.cols = d.cols;
    a.TC = d.TC;
    a.tiles = d.tiles;
    a.trace_offset = 0;
    a.reverse_order = 0;
    a.orient = ORIENT_FWD;
    a.ws_tr = ws_tr + d.tr_off;
    a.ws_gr = GRAD ? ws_gr + d.gr_off : nullptr;
    a.ckpt = nullptr;
    a.ckpt_interval = 0;
    a.nck = 0;
    if (GRAD)
      tile_adjoint_body(a, 0, it.y, smem);
    else
      tile_forward_body<false, true>(a, 0, it.y, smem);
    __syncthreads();
  }
}

__global__ void k_ragged_finish(const InstDesc* __restrict__ desc, const double2* __restrict__ ws_tr,
                                const double2* __restrict__ ws_gr, int variant, double* __restrict__ cost,
                                double* __restrict__ grad) {
  const InstDesc d = desc[blockIdx.x];
  double2 tr = make_double2(0.0, 0.0);
  for (int t = 0; t < d.tiles; t++) {
    double2 v = ws_tr[d.tr_off + t];
    tr.x += v.x;
    tr.y += v.y;
  }
  const double dc = d.cols;
  if (blockIdx.y == 0 && threadIdx.x == 0) {
    double f;
    if (variant == SQG_FROBENIUS_NORM) {
      f = 1.0 - tr.x / dc;
    } else if (variant == SQG_HILBERT_SCHMIDT_TEST) {
      double q = 1.0 / dc;
      f = 1.0 - q * q * (tr.x * tr.x + tr.y * tr.y);
    } else {
      f = 1.0 - ((tr.x * tr.x + tr.y * tr.y) / dc + 1) / (dc + 1);
    }
    cost[blockIdx.x] = f;
  }
  if (!grad) return;
  const int p = blockIdx.y * blockDim.x + threadIdx.x;
  if (p >= d.P) return;
  double2 dt = make_double2(0.0, 0.0);
  for (int t = 0; t < d.tiles; t++) {
    double2 v = ws_gr[d.gr_off + (long long)t * d.P + p];
    dt.x += v.x;
    dt.y += v.y;
  }
  double gv;
  if (variant == SQG_FROBENIUS_NORM) {
    gv = (1.0 - dt.x / dc) - 1.0;
  } else if (variant == SQG_HILBERT_SCHMIDT_TEST) {
    double q = 1.0 / dc;
    gv = -2.0 * q * q * tr.x * dt.x - 2.0 * q * q * tr.y * dt.y;
  } else {
    gv = -2.0 / dc / (dc + 1) * tr.x * dt.x - 2.0 / dc / (dc + 1) * tr.y * dt.y;
  }
  grad[d.theta_off + p] = gv;
}

int cerr(cudaError_t e, const char* where) {
  return e == cudaSuccess ? SQG_OK : set_error(SQG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

void free_batch(sqg_ragged_batch* r) {
  if (!r) return;
  cudaFree(r->d_desc);
  cudaFree(r->d_items);
  cudaFree(r->d_gate_map);
  delete r;
}

}  // namespace

extern "C" {

int sqg_ragged_create(const sqg_circuit* const* circuits, const int* cols, int count, int with_grad,
                      const int* tile_cols, sqg_ragged_batch** out) {
  if (!out) return set_error(SQG_ERR_INVALID_ARGUMENT, "null output handle");
  *out = nullptr;
  if (!circuits || !cols || count <= 0 || count > 65535)
    return set_error(SQG_ERR_INVALID_ARGUMENT, "need 1..65535 circuits and target widths");
  auto* r = new sqg_ragged_batch();
  r->count = count;
  r->with_grad = with_grad ? 1 : 0;
  cudaGetDevice(&r->device);
  std::vector<InstDesc> desc(count);
  std::vector<int2> gate_map;
  std::vector<std::pair<double, int2>> work;
  long long th = 0, tg = 0;
  size_t smem = 0;
  for (int i = 0; i < count; i++) {
    const sqg_circuit* c = circuits[i];
    if (!c || c->device != r->device || cols[i] <= 0 || cols[i] > (c ? c->N : 0)) {
      free_batch(r);
      return set_error(SQG_ERR_INVALID_ARGUMENT, "instance " + std::to_string(i) + ": bad circuit or target width");
    }
    if (c->n > 13) {
      free_batch(r);
      return set_error(SQG_ERR_UNSUPPORTED, "ragged batches hold whole columns on chip: qbit_num <= 13");
    }
    if (with_grad && c->n > 12) {
      free_batch(r);
      return set_error(SQG_ERR_UNSUPPORTED, "gradient supports qbit_num <= 12");
    }
    InstDesc& d = desc[i];
    d.gates = c->d_gates;
    d.L = c->L; d.P = c->P; d.n = c->n; d.N = c->N; d.cols = cols[i];
    const size_t per = (size_t)c->N * sizeof(double2) * (with_grad ? 2 : 1);
    int tc;
    if (tile_cols && tile_cols[i] > 0) {
      tc = std::min(tile_cols[i], cols[i]);
    } else {
      tc = (int)std::max<size_t>(1, (size_t)100 * 1024 / per);
      int p2 = 1;
      while (p2 * 2 <= tc) p2 *= 2;
      tc = std::min(p2, cols[i]);
    }
    if (tile_smem_bytes(tc, c->N, with_grad) > 220 * 1024) {
      free_batch(r);
      return set_error(SQG_ERR_UNSUPPORTED, "instance " + std::to_string(i) + ": tile does not fit in shared memory");
    }
    d.TC = tc;
    d.tiles = (cols[i] + tc - 1) / tc;
    d.theta_off = th;
    d.target_off = tg;
    d.gm_off = r->total_gm;
    d.sc_off = r->total_sc;
    d.tr_off = r->total_tr;
    d.gr_off = r->total_gr;
    r->theta_off.push_back(th);
    r->target_off.push_back(tg);
    th += c->P;
    tg += (long long)c->N * cols[i];
    r->total_gm += std::max(c->L, 1);
    r->total_sc += std::max(c->P, 1);
    r->total_tr += d.tiles;
    if (with_grad) r->total_gr += (long long)d.tiles * std::max(c->P, 1);
    r->maxP = std::max(r->maxP, c->P);
    smem = std::max(smem, tile_smem_bytes(tc, c->N, with_grad));
    for (int g = 0; g < c->L; g++) gate_map.push_back(make_int2(i, g));
    const double w = (double)std::max(c->L, 1) * c->N * tc;
    for (int t = 0; t < d.tiles; t++) work.push_back({w, make_int2(i, t)});
  }
  r->theta_off.push_back(th);
  r->target_off.push_back(tg);
  std::stable_sort(work.begin(), work.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
  std::vector<int2> items(work.size());
  for (size_t k = 0; k < work.size(); k++) items[k] = work[k].second;
  r->n_items = (int)items.size();
  r->total_gates = (int)gate_map.size();
  r->smem = smem;
  r->off_gm = 256;
  r->off_sc = a256(r->off_gm + sizeof(GateMat) * r->total_gm);
  r->off_tr = a256(r->off_sc + sizeof(double2) * r->total_sc);
  r->off_gr = a256(r->off_tr + sizeof(double2) * r->total_tr);
  r->ws_bytes = a256(r->off_gr + sizeof(double2) * std::max<long long>(r->total_gr, 1));
  cudaError_t e = cudaMalloc(&r->d_desc, sizeof(InstDesc) * count);
  if (e == cudaSuccess) e = cudaMalloc(&r->d_items, sizeof(int2) * std::max<size_t>(items.size(), 1));
  if (e == cudaSuccess) e = cudaMalloc(&r->d_gate_map, sizeof(int2) * std::max<size_t>(gate_map.size(), 1));
  if (e == cudaSuccess) e = cudaMemcpy(r->d_desc, desc.data(), sizeof(InstDesc) * count, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !items.empty())
    e = cudaMemcpy(r->d_items, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !gate_map.empty())
    e = cudaMemcpy(r->d_gate_map, gate_map.data(), sizeof(int2) * gate_map.size(), cudaMemcpyHostToDevice);
  // kernel attributes are set here, at planning time and to the device's opt-in maximum
  // (the attribute is per kernel, shared by every batch), so that launches can be captured
  // in CUDA graphs
  int optin = 0;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, r->device);
  if (e == cudaSuccess && smem + 64 > (size_t)optin) {
    free_batch(r);
    return set_error(SQG_ERR_UNSUPPORTED, "work item does not fit in shared memory");
  }
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_ragged_tiles<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - 64);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_ragged_tiles<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - 64);
  int per_sm = 0, sms = 0;
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, with_grad ? k_ragged_tiles<true> : k_ragged_tiles<false>, kRaggedThreads, smem);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, r->device);
  if (e != cudaSuccess) {
    int st = cerr(e, "sqg_ragged_create");
    free_batch(r);
    return st;
  }
  r->grid = std::max(1, std::min(r->n_items, std::max(per_sm, 1) * sms));
  *out = r;
  return SQG_OK;
}

int sqg_ragged_destroy(sqg_ragged_batch* r) {
  free_batch(r);
  return SQG_OK;
}

size_t sqg_ragged_workspace_bytes(const sqg_ragged_batch* r) { return r ? r->ws_bytes : 0; }

int sqg_ragged_layout(const sqg_ragged_batch* r, long long* theta_offsets, long long* target_offsets) {
  if (!r) return set_error(SQG_ERR_INVALID_ARGUMENT, "null batch");
  for (int i = 0; i <= r->count; i++) {
    if (theta_offsets) theta_offsets[i] = r->theta_off[i];
    if (target_offsets) target_offsets[i] = r->target_off[i];
  }
  return SQG_OK;
}

int sqg_ragged_cost_grad(const sqg_ragged_batch* r, const double* theta, const void* targets, int variant,
                         double* cost, double* grad, void* workspace, size_t ws_bytes, void* stream) {
  if (!r || !targets || !cost) return set_error(SQG_ERR_INVALID_ARGUMENT, "null batch, targets or cost");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != r->device) return set_error(SQG_ERR_INVALID_ARGUMENT, "batch belongs to another device");
  if (variant != SQG_FROBENIUS_NORM && variant != SQG_HILBERT_SCHMIDT_TEST && variant != SQG_INFIDELITY)
    return set_error(SQG_ERR_UNSUPPORTED, "cost function variant not implemented by the engine");
  if (grad && !r->with_grad) return set_error(SQG_ERR_INVALID_ARGUMENT, "batch was planned without gradients");
  if (!workspace || ws_bytes < r->ws_bytes)
    return set_error(SQG_ERR_WORKSPACE, "workspace too small: need " + std::to_string(r->ws_bytes));
  if (r->theta_off.back() > 0 && !theta) return set_error(SQG_ERR_INVALID_ARGUMENT, "null parameter array");
  cudaStream_t s = (cudaStream_t)stream;
  char* ws = (char*)workspace;
  int* counter = (int*)ws;
  GateMat* gm = (GateMat*)(ws + r->off_gm);
  double2* sc = (double2*)(ws + r->off_sc);
  double2* tr = (double2*)(ws + r->off_tr);
  double2* gr = (double2*)(ws + r->off_gr);
  int st;
  if ((st = cerr(cudaMemsetAsync(counter, 0, sizeof(int), s), "cudaMemsetAsync"))) return st;
  if (r->total_gates > 0) {
    k_ragged_prep<<<(r->total_gates + 127) / 128, 128, 0, s>>>(r->d_desc, r->d_gate_map, r->total_gates, theta, gm, sc);
    if ((st = cerr(cudaGetLastError(), "k_ragged_prep"))) return st;
  }
  const bool g = grad != nullptr;
  if (g)
    k_ragged_tiles<true><<<r->grid, kRaggedThreads, r->smem, s>>>(r->d_desc, r->d_items, r->n_items, counter,
                                                                  (const double2*)targets, gm, sc, tr, gr);
  else
    k_ragged_tiles<false><<<r->grid, kRaggedThreads, r->smem, s>>>(r->d_desc, r->d_items, r->n_items, counter,
                                                                   (const double2*)targets, gm, sc, tr, gr);
  if ((st = cerr(cudaGetLastError(), "k_ragged_tiles"))) return st;
  dim3 fgrid(r->count, g ? (r->maxP + 127) / 128 : 1);
  k_ragged_finish<<<fgrid, 128, 0, s>>>(r->d_desc, tr, gr, variant, cost, g ? grad : nullptr);
  return cerr(cudaGetLastError(), "k_ragged_finish");
}

}  // extern "C"
