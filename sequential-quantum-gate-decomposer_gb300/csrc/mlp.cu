// Kernels of the learned initialiser (an MLP mapping a target unitary to starting angles):
// BF16 GEMM with FP32 accumulation on the tensor cores, fused bias/ReLU epilogues, the
// backward-pass helpers, the angle head and Adam.  The initialiser has no counterpart in
// SQUANDER; it only proposes start points for the decomposition kernels, whose FP64 cost
// decides every result.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>

#include "../../include/sqg.h"
#include "handle.h"

namespace {

constexpr int BM = 64, BN = 64, BK = 32, PAD = 8;

__device__ __forceinline__ unsigned pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return (unsigned)__bfloat16_as_ushort(lo) | ((unsigned)__bfloat16_as_ushort(hi) << 16);
}

// C[M][N] = sum_k A'[m][k] B'[k][n] (+ bias[n], optional ReLU), FP32 accumulation.
// A' = A (row-major M x K, lda) or A^T (A stored K x M) when TA; B' = B (row-major K x N)
// or B^T (B stored N x K) when TB.  Tiles of 64 x 64 x 32 staged in shared memory
// (k-contiguous for both operands), 4 warps each computing 32 x 32 with
// mma.sync.m16n8k16 (bf16 in, f32 accumulate).
template <bool TA, bool TB>
__global__ void __launch_bounds__(128) k_gemm_bf16(int M, int N, int K, const __nv_bfloat16* __restrict__ A, int lda,
                                                   const __nv_bfloat16* __restrict__ B, int ldb, float* __restrict__ C,
                                                   int ldc, const float* __restrict__ bias, int relu,
                                                   __nv_bfloat16* __restrict__ Cb, int beta_accumulate) {
  __shared__ __align__(16) __nv_bfloat16 As[BM][BK + PAD];
  __shared__ __align__(16) __nv_bfloat16 Bs[BN][BK + PAD];
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int gid = lane >> 2, tig = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[i][j][q] = 0.f;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  for (int k0 = 0; k0 < K; k0 += BK) {
    for (int e = threadIdx.x; e < BM * BK; e += blockDim.x) {
      int r, kk;
      if (TA) {  // consecutive threads walk m (contiguous in memory)
        r = e % BM;
        kk = e / BM;
      } else {
        r = e / BK;
        kk = e % BK;
      }
      int gm = m0 + r, gk = k0 + kk;
      __nv_bfloat16 v = zero;
      if (gm < M && gk < K) v = TA ? A[(long long)gk * lda + gm] : A[(long long)gm * lda + gk];
      As[r][kk] = v;
    }
    for (int e = threadIdx.x; e < BN * BK; e += blockDim.x) {
      int r, kk;
      if (TB) {
        r = e / BK;
        kk = e % BK;
      } else {
        r = e % BN;
        kk = e / BN;
      }
      int gn = n0 + r, gk = k0 + kk;
      __nv_bfloat16 v = zero;
      if (gn < N && gk < K) v = TB ? B[(long long)gn * ldb + gk] : B[(long long)gk * ldb + gn];
      Bs[r][kk] = v;
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < BK; ks += 16) {
      unsigned af[2][4], bfr[4][2];
#pragma unroll
      for (int i = 0; i < 2; i++) {
        int r = wm + i * 16 + gid;
        af[i][0] = pack2(As[r][ks + 2 * tig], As[r][ks + 2 * tig + 1]);
        af[i][1] = pack2(As[r + 8][ks + 2 * tig], As[r + 8][ks + 2 * tig + 1]);
        af[i][2] = pack2(As[r][ks + 2 * tig + 8], As[r][ks + 2 * tig + 9]);
        af[i][3] = pack2(As[r + 8][ks + 2 * tig + 8], As[r + 8][ks + 2 * tig + 9]);
      }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        int c = wn + j * 8 + gid;
        bfr[j][0] = pack2(Bs[c][ks + 2 * tig], Bs[c][ks + 2 * tig + 1]);
        bfr[j][1] = pack2(Bs[c][ks + 2 * tig + 8], Bs[c][ks + 2 * tig + 9]);
      }
#pragma unroll
      for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
          asm volatile(
              "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
              "{%0,%1,%2,%3};\n"
              : "+f"(acc[i][j][0]), "+f"(acc[i][j][1]), "+f"(acc[i][j][2]), "+f"(acc[i][j][3])
              : "r"(af[i][0]), "r"(af[i][1]), "r"(af[i][2]), "r"(af[i][3]), "r"(bfr[j][0]), "r"(bfr[j][1]));
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int q = 0; q < 4; q++) {
        int r = m0 + wm + i * 16 + gid + (q >= 2 ? 8 : 0);
        int c = n0 + wn + j * 8 + 2 * tig + (q & 1);
        if (r < M && c < N) {
          float v = acc[i][j][q];
          if (beta_accumulate && C) v += C[(long long)r * ldc + c];
          if (bias) v += bias[c];
          if (relu) v = fmaxf(v, 0.f);
          if (C) C[(long long)r * ldc + c] = v;
          if (Cb) Cb[(long long)r * ldc + c] = __float2bfloat16(v);
        }
      }
}

__global__ void k_f32_to_bf16(const float* __restrict__ x, __nv_bfloat16* __restrict__ y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16(x[i]);
}

// dZ = dA * (Z > 0) in place on dA (fp32), plus a bf16 copy for the next GEMMs.
__global__ void k_relu_backward(float* __restrict__ dA, const float* __restrict__ Z, __nv_bfloat16* __restrict__ dZb,
                                long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float v = Z[i] > 0.f ? dA[i] : 0.f;
    dA[i] = v;
    dZb[i] = __float2bfloat16(v);
  }
}

// db[n] = sum_m dZ[m][n] (fixed order over m).
__global__ void k_col_sum(const float* __restrict__ dZ, int M, int N, float* __restrict__ db) {
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int m = 0; m < M; m++) s += dZ[(long long)m * N + n];
  db[n] = s;
}

// Adam on fp32 master weights; refreshes the bf16 working copy.
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       __nv_bfloat16* __restrict__ wb, long long n, float lr, float b1, float b2, float eps, float c1,
                       float c2, float wd) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float gi = g[i] + wd * w[i];
    float mi = b1 * m[i] + (1.f - b1) * gi;
    float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
  }
}

// Angle head: the network emits (c_k, s_k) per angle; theta_k = atan2(s_k, c_k).
//   mode 0: theta only;  mode 1: supervised loss sum_k |(c,s) - (cos t*, sin t*)|^2 / P and its
//   gradient;  mode 2: chain rule of an external dL/dtheta (e.g. the decomposition cost
//   gradient) through atan2.  out_grad has the head's layout (M x 2P).
__global__ void k_angle_head(const float* __restrict__ out, int M, int P, double* __restrict__ theta,
                             const double* __restrict__ target_or_dtheta, int mode, float scale,
                             float* __restrict__ out_grad, float* __restrict__ loss_rows) {
  int m = blockIdx.x;
  if (m >= M) return;
  float acc = 0.f;
  for (int k = threadIdx.x; k < P; k += blockDim.x) {
    float c = out[(long long)m * 2 * P + 2 * k], s = out[(long long)m * 2 * P + 2 * k + 1];
    double th = atan2((double)s, (double)c);
    if (theta) theta[(long long)m * P + k] = th;
    if (mode == 1) {
      double t = target_or_dtheta[(long long)m * P + k];
      float dc = c - (float)cos(t), ds = s - (float)sin(t);
      acc += dc * dc + ds * ds;
      out_grad[(long long)m * 2 * P + 2 * k] = 2.f * dc * scale;
      out_grad[(long long)m * 2 * P + 2 * k + 1] = 2.f * ds * scale;
    } else if (mode == 2) {
      float r2 = c * c + s * s + 1e-12f;
      float gth = (float)target_or_dtheta[(long long)m * P + k];
      out_grad[(long long)m * 2 * P + 2 * k] = -s / r2 * gth * scale;
      out_grad[(long long)m * 2 * P + 2 * k + 1] = c / r2 * gth * scale;
    }
  }
  if (mode == 1 && loss_rows) {
    __shared__ float red[32];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      float t = 0.f;
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
      loss_rows[m] = t / P;
    }
  }
}

// Network input: Re/Im of a batch of rows x cols complex128 targets, interleaved, as bf16.
__global__ void k_features(const double2* __restrict__ U, long long n_complex, __nv_bfloat16* __restrict__ x) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_complex;
       i += (long long)gridDim.x * blockDim.x) {
    double2 u = U[i];
    x[2 * i] = __float2bfloat16((float)u.x);
    x[2 * i + 1] = __float2bfloat16((float)u.y);
  }
}

int grid_for(long long n) { return (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096); }

int launch_status(const char* where) {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SQG_OK : sqg::set_error(SQG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

}  // namespace

extern "C" {

int sqg_mlp_gemm_bf16(int M, int N, int K, const void* A, int lda, int transA, const void* B, int ldb, int transB,
                      float* C, int ldc, const float* bias, int relu, void* C_bf16, int accumulate, void* stream) {
  if (M <= 0 || N <= 0 || K <= 0 || !A || !B || (!C && !C_bf16) || (accumulate && !C))
    return sqg::set_error(SQG_ERR_INVALID_ARGUMENT, "bad GEMM arguments");
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
  cudaStream_t s = (cudaStream_t)stream;
  auto a = (const __nv_bfloat16*)A;
  auto b = (const __nv_bfloat16*)B;
  auto cb = (__nv_bfloat16*)C_bf16;
  if (!transA && transB)
    k_gemm_bf16<false, true><<<grid, 128, 0, s>>>(M, N, K, a, lda, b, ldb, C, ldc, bias, relu, cb, accumulate);
  else if (!transA && !transB)
    k_gemm_bf16<false, false><<<grid, 128, 0, s>>>(M, N, K, a, lda, b, ldb, C, ldc, bias, relu, cb, accumulate);
  else if (transA && !transB)
    k_gemm_bf16<true, false><<<grid, 128, 0, s>>>(M, N, K, a, lda, b, ldb, C, ldc, bias, relu, cb, accumulate);
  else
    k_gemm_bf16<true, true><<<grid, 128, 0, s>>>(M, N, K, a, lda, b, ldb, C, ldc, bias, relu, cb, accumulate);
  return launch_status("k_gemm_bf16");
}

int sqg_mlp_to_bf16(const float* x, void* y, long long n, void* stream) {
  if (!x || !y || n < 0) return sqg::set_error(SQG_ERR_INVALID_ARGUMENT, "bad conversion arguments");
  if (n == 0) return SQG_OK;
  k_f32_to_bf16<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(x, (__nv_bfloat16*)y, n);
  return launch_status("k_f32_to_bf16");
}

int sqg_mlp_relu_backward(float* dA, const float* Z, void* dZ_bf16, long long n, void* stream) {
  if (!dA || !Z || !dZ_bf16 || n <= 0) return sqg::set_error(SQG_ERR_INVALID_ARGUMENT, "bad ReLU arguments");
  k_relu_backward<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(dA, Z, (__nv_bfloat16*)dZ_bf16, n);
  return launch_status("k_relu_backward");
}

int sqg_mlp_col_sum(const float* dZ, int M, int N, float* db, void* stream) {
  if (!dZ || !db || M <= 0 || N <= 0) return sqg::set_error(SQG_ERR_INVALID_ARGUMENT, "bad column-sum arguments");
  k_col_sum<<<(N + 127) / 128, 128, 0, (cudaStream_t)stream>>>(dZ, M, N, db);
  return launch_status("k_col_sum");
}

int sqg_mlp_adam(float* w, const float* g, float* m, float* v, void* w_bf16, long long n, float lr, float beta1,
                 float beta2, float eps, int step, float weight_decay, void* stream) {
  if (!w || !g || !m || !v || n <= 0 || step < 1) return sqg::set_error(SQG_ERR_INVALID_ARGUMENT, "bad Adam arguments");
  float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  k_adam<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(w, g, m, v, (__nv_bfloat16*)w_bf16, n, lr, beta1, beta2, eps,
                                                       c1, c2, weight_decay);
  return launch_status("k_adam");
}

int sqg_mlp_angle_head(const float* out, int M, int P, double* theta, const double* target_or_dtheta, int mode,
                       float scale, float* out_grad, float* loss_rows, void* stream) {
  if (!out || M <= 0 || P <= 0 || mode < 0 || mode > 2 || (mode > 0 && (!target_or_dtheta || !out_grad)))
    return sqg::set_error(SQG_ERR_INVALID_ARGUMENT, "bad angle-head arguments");
  k_angle_head<<<M, 128, 0, (cudaStream_t)stream>>>(out, M, P, theta, target_or_dtheta, mode, scale, out_grad,
                                                    loss_rows);
  return launch_status("k_angle_head");
}

int sqg_mlp_features(const void* U, long long n_complex, void* x_bf16, void* stream) {
  if (!U || !x_bf16 || n_complex <= 0) return sqg::set_error(SQG_ERR_INVALID_ARGUMENT, "bad feature arguments");
  k_features<<<grid_for(n_complex), 256, 0, (cudaStream_t)stream>>>((const double2*)U, n_complex,
                                                                   (__nv_bfloat16*)x_bf16);
  return launch_status("k_features");
}

}  // extern "C"
