// BF16 GEMM on the 5th-generation tensor cores (tcgen05.mma, accumulator in TMEM) with
// operands staged by TMA (cp.async.bulk.tensor, 128-byte swizzle): the learned
// initialiser's layer GEMMs.  C[M][N] = A[M][K] * B[N][K]^T (+ bias[n], optional ReLU),
// both operands K-major bf16, FP32 accumulation; results as fp32 and/or bf16.
//
// One CTA computes a 128 x TN tile (TN = 256 where N is a multiple of 256, else 128): warp 0
// allocates TN TMEM columns; one thread of warp 0 issues the TMA loads into a ring of four
// stages (128 x 64 of A, TN x 64 of B) and waits only for a stage's "empty" barrier, one
// thread of warp 1 issues the MMAs (4 x 128 x TN x 16 per stage) and commits each stage to
// that barrier; finally the four warps read their 32 TMEM lanes each (32x32b loads) into a
// padded shared-memory tile and store it row by row (coalesced), with the bias / ReLU
// epilogue.  Every mbarrier wait is bounded: on a time-out the CTA records an error code,
// drains its own copies and MMAs (again bounded), frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/sqg.h"
#include "handle.h"

namespace {

constexpr int TM = 128, TK = 64;
__host__ __device__ constexpr int stage_bytes(int TN) { return (TM + TN) * TK * 2; }
constexpr unsigned kSpinLimit = 1u << 24;

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// Bounded wait for the phase with the given parity; returns false on time-out.  Polls with the
// non-blocking test_wait: try_wait may suspend the thread for a hardware-chosen interval, which
// a producer or MMA thread that arrives just before the phase completes would pay every k-step.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  for (unsigned i = 0; i < kSpinLimit; i++) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(unsigned dst, const CUtensorMap* map, int x, int y, unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"((unsigned long long)map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms 1024 bytes apart.
__device__ __forceinline__ unsigned long long smem_desc(unsigned addr) {
  unsigned long long d = 0;
  d |= (unsigned long long)((addr >> 4) & 0x3FFF);          // start address
  d |= (unsigned long long)(0) << 16;                        // leading byte offset (unused)
  d |= (unsigned long long)((1024 >> 4) & 0x3FFF) << 32;     // stride byte offset
  d |= (unsigned long long)1 << 46;                          // descriptor version
  d |= (unsigned long long)2 << 61;                          // 128-byte swizzle
  return d;
}

// Instruction descriptor of kind::f16: bf16 A and B (K-major), fp32 accumulator, M x N.
__host__ __device__ constexpr unsigned instr_desc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}

template <int TN, int STAGES>
__global__ void __launch_bounds__(128, 1) k_gemm_tc(const __grid_constant__ CUtensorMap mapA,
                                                     const __grid_constant__ CUtensorMap mapB, int M, int N, int K,
                                                     float* __restrict__ C, int ldc, const float* __restrict__ bias,
                                                     int relu, __nv_bfloat16* __restrict__ Cb, int* err) {
  constexpr int STAGE_BYTES = stage_bytes(TN);
  constexpr int EPI_LD = TN + 1;  // fp32 epilogue tile row (odd: no bank conflicts)
  static_assert(TM * EPI_LD * 4 <= STAGES * STAGE_BYTES, "the epilogue tile reuses the stage buffers");
  extern __shared__ __align__(1024) unsigned char dsmem[];
  // 1024-byte alignment for the swizzled tiles
  unsigned char* base = (unsigned char*)(((unsigned long long)dsmem + 1023) & ~1023ull);
  __shared__ __align__(8) unsigned long long bar_full[STAGES], bar_empty[STAGES], bar_final;
  __shared__ unsigned tmem_base_s;
  __shared__ int failed_s, issued_s, consumed_s, final_ok_s;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
  const int ktiles = (K + TK - 1) / TK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(smem_u32(&bar_full[s]), 1);
      mbar_init(smem_u32(&bar_empty[s]), 1);
    }
    mbar_init(smem_u32(&bar_final), 1);
    failed_s = 0;
    issued_s = 0;
    consumed_s = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                 "r"(TN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const unsigned tmem = tmem_base_s;
  const unsigned idesc = instr_desc(TM, TN);
  volatile int* failed = &failed_s;

  if (warp == 0 && lane == 0) {
    // TMA producer: fills stage s again once the MMAs that read it have completed
    int issued = 0;
    for (int kt = 0; kt < ktiles && !*failed; kt++) {
      const int s = kt % STAGES;
      if (kt >= STAGES && !mbar_wait(smem_u32(&bar_empty[s]), ((kt / STAGES) - 1) & 1)) {
        *failed = 1;
        break;
      }
      const unsigned sa = smem_u32(base + s * STAGE_BYTES), sb = sa + TM * TK * 2;
      const unsigned bf = smem_u32(&bar_full[s]);
      mbar_expect_tx(bf, STAGE_BYTES);
      tma_load_2d(sa, &mapA, kt * TK, m0, bf);
      tma_load_2d(sb, &mapB, kt * TK, n0, bf);
      issued++;
    }
    issued_s = issued;
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: four K = 16 MMAs per stage, each stage committed to its empty barrier
    int consumed = 0;
    for (int kt = 0; kt < ktiles && !*failed; kt++) {
      const int s = kt % STAGES;
      if (!mbar_wait(smem_u32(&bar_full[s]), (kt / STAGES) & 1)) {
        *failed = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const unsigned sa = smem_u32(base + s * STAGE_BYTES), sb = sa + TM * TK * 2;
#pragma unroll
      for (int k = 0; k < TK / 16; k++) {
        unsigned long long da = smem_desc(sa + k * 32), db = smem_desc(sb + k * 32);
        unsigned acc = (kt > 0 || k > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(da), "l"(db), "r"(idesc), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&bar_empty[s]))
                   : "memory");
      consumed++;
    }
    consumed_s = consumed;
    // completion of every MMA issued above (also after a time-out)
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(&bar_final))
                 : "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (failed_s) {
      atomicExch(err, 1);
      // drain: wait (bounded) for the copies issued but not consumed by an MMA
      for (int kt = consumed_s; kt < issued_s; kt++) mbar_wait(smem_u32(&bar_full[kt % STAGES]), (kt / STAGES) & 1);
    }
    final_ok_s = mbar_wait(smem_u32(&bar_final), 0) ? 1 : 0;
    if (!final_ok_s) atomicExch(err, 2);
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (final_ok_s && !failed_s) {
    // every MMA has completed: the stage buffers hold the fp32 tile for coalesced stores
    float* epi = reinterpret_cast<float*>(base);
    const int r = warp * 32 + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < TN; c0 += 32) {
      unsigned v[32];
      const unsigned taddr = tmem + ((unsigned)(warp * 32) << 16) + c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,"
          "%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
            "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
            "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int j = 0; j < 32; j++) epi[r * EPI_LD + c0 + j] = __uint_as_float(v[j]);
    }
    __syncthreads();
    for (int rr = warp; rr < TM; rr += 4) {
      const int row = m0 + rr;
      if (row >= M) continue;
      for (int c = lane; c < TN; c += 32) {
        const int col = n0 + c;
        if (col >= N) continue;
        float x = epi[rr * EPI_LD + c];
        if (bias) x += bias[col];
        if (relu) x = fmaxf(x, 0.f);
        if (C) C[(long long)row * ldc + col] = x;
        if (Cb) Cb[(long long)row * ldc + col] = __float2bfloat16(x);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TN));
}

// bf16 transpose: out[c][r] = in[r][c] (rows x cols, row strides in elements).
__global__ void k_transpose_bf16(const __nv_bfloat16* __restrict__ in, int rows, int cols, int ld_in,
                                 __nv_bfloat16* __restrict__ out, int ld_out) {
  __shared__ __nv_bfloat16 t[32][33];
  int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int r = by + j, c = bx + threadIdx.x;
    if (r < rows && c < cols) t[j][threadIdx.x] = in[(long long)r * ld_in + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int c = bx + j, r = by + threadIdx.x;
    if (c < cols && r < rows) out[(long long)c * ld_out + r] = t[threadIdx.x][j];
  }
}

typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
  static EncodeTiled fn = nullptr;
  static std::once_flag once;
  std::call_once(once, []() {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiled)p;
  });
  return fn;
}

// 2-D K-major bf16 tensor map: rows x K elements, row stride ld elements, box 64 x box_rows.
int make_map(CUtensorMap* map, const void* ptr, int rows, int K, int ld, int box_rows) {
  EncodeTiled enc = encode_fn();
  if (!enc) return sqg::set_error(SQG_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {TK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return sqg::set_error(SQG_ERR_INVALID_ARGUMENT, "cuTensorMapEncodeTiled failed");
  return SQG_OK;
}

template <int TN, int STAGES>
int gemm_launch(int M, int N, int K, const void* A, int lda, const void* B, int ldb, float* C, int ldc,
                const float* bias, int relu, void* C_bf16, int* err_dev, void* stream) {
  CUtensorMap ma, mb;
  int st;
  if ((st = make_map(&ma, A, M, K, lda, TM))) return st;
  if ((st = make_map(&mb, B, N, K, ldb, TN))) return st;
  const size_t smem = (size_t)STAGES * stage_bytes(TN) + 1024;
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [&]() {
    attr = cudaFuncSetAttribute(k_gemm_tc<TN, STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  });
  if (attr != cudaSuccess) return sqg::set_error(SQG_ERR_CUDA, cudaGetErrorString(attr));
  dim3 grid((N + TN - 1) / TN, (M + TM - 1) / TM);
  k_gemm_tc<TN, STAGES><<<grid, 128, smem, (cudaStream_t)stream>>>(ma, mb, M, N, K, C, ldc, bias, relu,
                                                                   (__nv_bfloat16*)C_bf16, err_dev);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SQG_OK : sqg::set_error(SQG_ERR_CUDA, std::string("k_gemm_tc: ") + cudaGetErrorString(e));
}

}  // namespace

extern "C" {

int sqg_mlp_gemm_tc(int M, int N, int K, const void* A, int lda, const void* B, int ldb, float* C, int ldc,
                    const float* bias, int relu, void* C_bf16, int* err_dev, void* stream) {
  if (M <= 0 || N <= 0 || K <= 0 || !A || !B || (!C && !C_bf16) || !err_dev)
    return sqg::set_error(SQG_ERR_INVALID_ARGUMENT, "bad GEMM arguments");
  if (K % 8 || lda % 8 || ldb % 8 || ((unsigned long long)A & 15) || ((unsigned long long)B & 15))
    return sqg::set_error(SQG_ERR_INVALID_ARGUMENT,
                          "tensor-core GEMM needs 16-byte aligned operands and K, lda, ldb multiples of 8");
  // 128 x 256 tiles (one 128 x 256 x 16 MMA per K = 16 step, B read once per 256 columns) where
  // N fills them; 128 x 128 for narrow or ragged N, where a 256-wide tile would idle columns
  if (N % 256 == 0) return gemm_launch<256, 4>(M, N, K, A, lda, B, ldb, C, ldc, bias, relu, C_bf16, err_dev, stream);
  return gemm_launch<128, 4>(M, N, K, A, lda, B, ldb, C, ldc, bias, relu, C_bf16, err_dev, stream);
}

int sqg_mlp_transpose_bf16(const void* in, int rows, int cols, int ld_in, void* out, int ld_out, void* stream) {
  if (!in || !out || rows <= 0 || cols <= 0) return sqg::set_error(SQG_ERR_INVALID_ARGUMENT, "bad transpose");
  dim3 grid((cols + 31) / 32, (rows + 31) / 32);
  k_transpose_bf16<<<grid, dim3(32, 8), 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)in, rows, cols, ld_in,
                                                                   (__nv_bfloat16*)out, ld_out);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SQG_OK : sqg::set_error(SQG_ERR_CUDA, cudaGetErrorString(e));
}

}  // extern "C"
