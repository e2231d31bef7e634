// BFGS with Powell's Z-matrix update for one target on one CTA: the building blocks shared by
// the batched decomposition kernel (decompose.cu: vectors in shared memory, one CTA per target)
// and the graph-driven single-target loop (loop.cu: vectors and Z in global memory).
//
// Restated from SQUANDER's BFGS_Powell (common/BFGS_Powell.cpp:194-446) and the maximal step
// of its line search (common/grad_descend.cpp:399-425).  Every routine is called by all threads
// of one CTA (blockDim.x a multiple of 32, at most kTileMaxThreads) and ends with a barrier
// where its results are read by other threads.
#pragma once
#include "tile.cuh"

namespace sqg {

// Z entries per load batch in the row and column passes.  4 since the evaluation of the batched
// decomposition kernel is no longer inlined: with it out of line, chunks of 4 gave 10060
// decompositions/s against 9536 with chunks of 8 (the same evaluation counts).
constexpr int kChunk = 4;
constexpr double kNumPrecision = 1.42e-14;  // grad_descend.cpp:37
constexpr double kTwoPi = 6.283185307179586476925286766559;

// Vectors of one BFGS target (P doubles each) and its Z matrix (P x P, row-major, held as
// Zs diag(cs)); redd: kTileMaxWarps * 8 doubles, scratch: kTileMaxWarps doubles.
struct BfgsVecs {
  double *Z, *x, *x0, *g, *g0, *gbest, *d, *delta, *gamma, *v, *vp, *cs, *ztg, *zs, *S, *sdv, *nz, *gtz;
  double *redd, *scratch;
};

// Accessors of the Z matrix.  ZMem: plain loads and stores (Z in shared memory, or global).
// ZKeepL2: Z in global memory, every load and store carrying an L2 evict_last policy, so
// that the matrices of the resident CTAs stay in L2 rather than being written back to HBM
// between the passes of one iteration.  The address must point to global memory.
struct ZMem {
  __device__ __forceinline__ double ld(const double* p) const { return *p; }
  __device__ __forceinline__ void st(double* p, double v) const { *p = v; }
};

struct ZKeepL2 {
  unsigned long long pol;
  __device__ __forceinline__ ZKeepL2() { asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol)); }
  __device__ __forceinline__ double ld(const double* p) const {
    double v;
    asm volatile("ld.global.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol) : "memory");
    return v;
  }
  __device__ __forceinline__ void st(double* p, double v) const {
    asm volatile("st.global.L2::cache_hint.f64 [%0], %1, %2;" ::"l"(p), "d"(v), "l"(pol) : "memory");
  }
};

static __device__ __forceinline__ double u01(unsigned long long k) {
  unsigned long long z = k + 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

static __device__ double dot(const double* a, const double* b, int P, double* scratch) {
  double s = 0.0;
  for (int i = threadIdx.x; i < P; i += blockDim.x) s = fma(a[i], b[i], s);
  return block_allsum(s, scratch);
}

// out[k] = sum_{k <= i < P} a[i] b[i] for every k, in a fixed order (a suffix scan inside
// each warp, then the totals of the later warps and of the later segments of blockDim
// entries).  Called by all threads; ends with a barrier.
static __device__ void block_suffix_dot(double* out, const double* a, const double* b, int P, double* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double carry = 0.0;
  for (int seg = (P - 1) / (int)blockDim.x; seg >= 0; seg--) {
    const int k = seg * blockDim.x + threadIdx.x;
    double v = k < P ? a[k] * b[k] : 0.0;
    for (int o = 1; o < 32; o <<= 1) {
      const double u = __shfl_down_sync(0xffffffffu, v, o);
      if (lane + o < 32) v += u;
    }
    __syncthreads();
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    double later = carry;
    for (int w = nw - 1; w > warp; w--) later += scratch[w];
    if (k < P) out[k] = v + later;
    if (seg > 0) {  // same order in every thread, so all threads carry the same value
      double t = carry;
      for (int w = nw - 1; w >= 0; w--) t += scratch[w];
      carry = t;
    }
  }
  __syncthreads();
}

// Maximum of an int over the CTA, returned to every thread.
static __device__ __forceinline__ int block_allmax_int(int v, double* scratch) {
  int* s = reinterpret_cast<int*>(scratch);
  v = __reduce_max_sync(0xffffffffu, v);
  const int nw = blockDim.x >> 5;
  if (nw == 1) return v;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
  __syncthreads();
  int t = s[0];
  for (int w = 1; w < nw; w++) t = max(t, s[w]);
  return t;
}

// BFGS_Powell::BFGS_iteration (BFGS_Powell.cpp:202-396) on the vectors of one target; returns
// the updated norm_Z.  On entry x, g are the accepted point and gradient, x0, g0 those the
// line search started from.
//
// Z is held as Zs diag(cs): column scalings are recorded in cs and folded into the next
// read of the column.  On entry sh.ztg = Z^T g0 and sh.zs = cs * ztg (this iteration's
// search direction); on exit they hold the same for the updated Z and the accepted
// gradient g, so the next direction needs no Z^T g pass.
//
// Only one pass reads Z before the rotation: v = Z^T g.  With Q the reference's Givens
// chain (Q^T ztg = |ztg| e_0), the reference's gTz = (Z Q)^T (g - g0) / dtg is, for the
// columns c >= 1 it uses, (Q^T v)_c / dtg, and after the rank-one update and the scaling
// by s_c, (Z_new^T g)_c = s_c ((Q^T v)_c - gTz_c (delta . g)); column 0 (delta / sqrt(dtg))
// is dotted with g directly.
//
// The chain itself is evaluated in closed form: with S_k = sum_{i>=k} z_i^2, m the last
// nonzero index of z = ztg, r_k = sqrt(S_k) (k < m) and r_m = z_m, the rotation at col
// (pairing col-1, col; col = m..1) has a = r_{col-1}, cos = z_{col-1} / a, sin = r_col / a,
// and the carry entering column col of a row y is sum_{i>=col} y_i z_i / r_col, so
//   y'_col = alpha_col * sum_{i>=col} y_i z_i - beta_col * y_{col-1},
//   alpha_col = z_{col-1} / (r_{col-1} r_col),  beta_col = r_col / r_{col-1}.
// Keeping alpha_col as the column's new scale leaves two FP64 operations per entry.
template <class ZA>
static __device__ double bfgs_update(int P, const BfgsVecs& sh, double norm_Z, const ZA& za) {
  double* Z = sh.Z;
  double red[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    const double de = sh.x[i] - sh.x0[i], ga = sh.g[i] - sh.g0[i];
    sh.delta[i] = de;
    sh.gamma[i] = ga;
    red[0] = fma(de, de, red[0]);
    red[1] = fma(sh.g0[i], de, red[1]);
    red[2] = fma(ga, de, red[2]);
    red[3] = fma(sh.g[i], de, red[3]);
  }
  for (int c = threadIdx.x; c < P; c += blockDim.x) {
    double s = 0.0;
#pragma unroll 8
    for (int r = 0; r < P; r++) s = fma(za.ld(Z + (long long)r * P + c), sh.g[r], s);
    sh.v[c] = s * sh.cs[c];
  }
  block_allsum_n(red, sh.redd);
  const double norm_delta = red[0], tmp = red[1], dgn = red[3];
  double dtg = red[2];
  if (dtg < fabs(tmp) * 0.1) {  // no update: Z^T g is v
    for (int c = threadIdx.x; c < P; c += blockDim.x) {
      sh.ztg[c] = sh.v[c];
      sh.zs[c] = sh.v[c] * sh.cs[c];
    }
    __syncthreads();
    return norm_Z;
  }
  dtg = fmax(kNumPrecision, dtg);
  block_suffix_dot(sh.S, sh.ztg, sh.ztg, P, sh.scratch);
  block_suffix_dot(sh.sdv, sh.v, sh.ztg, P, sh.scratch);
  int lnz = -1;
  for (int i = threadIdx.x; i < P; i += blockDim.x)
    if (sh.ztg[i] != 0.0) lnz = i;
  const int m = block_allmax_int(lnz, sh.scratch);
  for (int k = threadIdx.x; k <= m; k += blockDim.x) {
    const double r = k == m ? sh.ztg[m] : sqrt(sh.S[k]);
    sh.nz[k] = r;
    sh.S[k] = 1.0 / r;
  }
  __syncthreads();
  // per column: Q^T v (vp), the new scale alpha (nz), q = -beta cs_{col-1} / alpha (gtz)
  // and beta cs_{col-1} (sdv) for the three-operation form used when some alpha is 0
  bool zero_alpha = false;
  for (int col = threadIdx.x; col < P; col += blockDim.x) {
    if (col == 0) continue;
    if (col > m) {
      sh.vp[col] = sh.v[col];
      continue;
    }
    const double ir0 = sh.S[col - 1], ir1 = sh.S[col], zc = sh.ztg[col - 1];
    const double al = zc * ir0 * ir1, be = sh.nz[col] * ir0;
    sh.vp[col] = fma(al, sh.sdv[col], -be * sh.v[col - 1]);
    const double bc = be * sh.cs[col - 1];
    sh.sdv[col] = bc;
    sh.nz[col] = al;
    if (zc != 0.0)
      sh.gtz[col] = -bc / al;
    else
      zero_alpha = true;
  }
  zero_alpha = __syncthreads_or(zero_alpha);
  // Rows in chunks of kChunk columns: all loads of a chunk are issued before its stores,
  // so a row costs one memory round trip per chunk instead of one per column (a lone
  // CTA, as at the end of a batch, sees the full L2 latency).
  for (int r = threadIdx.x; r < P; r += blockDim.x) {
    double* row = Z + (long long)r * P;
    if (m < 1) break;
    double sd = 0.0, ycur = za.ld(row + m);
    for (int col = m; col >= 1; col -= kChunk) {
      double yp[kChunk], out[kChunk];
#pragma unroll
      for (int j = 0; j < kChunk; j++) yp[j] = col - 1 - j >= 0 ? za.ld(row + col - 1 - j) : 0.0;
      if (!zero_alpha) {
#pragma unroll
        for (int j = 0; j < kChunk; j++) {
          const int cc = max(col - j, 1);
          sd = fma(ycur, sh.zs[cc], sd);
          out[j] = fma(sh.gtz[cc], yp[j], sd);  // times alpha_cc (the column's scale)
          ycur = yp[j];
        }
      } else {
#pragma unroll
        for (int j = 0; j < kChunk; j++) {
          const int cc = max(col - j, 1);
          sd = fma(ycur, sh.zs[cc], sd);
          out[j] = fma(sh.nz[cc], sd, -sh.sdv[cc] * yp[j]);
          ycur = yp[j];
        }
      }
#pragma unroll
      for (int j = 0; j < kChunk; j++)
        if (col - j >= 1) za.st(row + col - j, out[j]);
    }
  }
  if (norm_Z < 0.0) {
    norm_Z = norm_delta / dtg;
  } else {
    double t = sqrt(norm_Z * norm_delta / dtg);
    norm_Z = fmin(norm_Z, t);
    norm_Z = fmax(norm_Z, t * 0.1);
  }
  const double isdt = 1.0 / sqrt(dtg), idtg = 1.0 / dtg;
  __syncthreads();
  double c0 = 0.0;
  for (int r = threadIdx.x; r < P; r += blockDim.x) {
    const double z0 = fabs(sh.delta[r]) > kNumPrecision ? sh.delta[r] * isdt : 0.0;
    za.st(Z + (long long)r * P, z0);
    c0 = fma(z0, sh.g[r], c0);
  }
  for (int col = threadIdx.x + 1; col <= m; col += blockDim.x) sh.cs[col] = zero_alpha ? 1.0 : sh.nz[col];
  c0 = block_allsum(c0, sh.scratch);
  __syncthreads();
  for (int c = threadIdx.x; c < P; c += blockDim.x) {
    if (c == 0) {
      sh.cs[0] = 1.0;
      sh.ztg[0] = c0;
      sh.zs[0] = c0;
      continue;
    }
    const double cs = sh.cs[c], gtz = sh.vp[c] * idtg, gc = gtz / cs;
    double s = 0.0;
    for (int r0 = 0; r0 < P; r0 += kChunk) {
      double zv[kChunk];
#pragma unroll
      for (int j = 0; j < kChunk; j++) zv[j] = r0 + j < P ? za.ld(Z + (long long)(r0 + j) * P + c) : 0.0;
#pragma unroll
      for (int j = 0; j < kChunk; j++) {
        if (r0 + j < P) {
          zv[j] = zv[j] - gc * sh.delta[r0 + j];
          s = fma(zv[j], zv[j], s);
        }
      }
#pragma unroll
      for (int j = 0; j < kChunk; j++)
        if (r0 + j < P) za.st(Z + (long long)(r0 + j) * P + c, zv[j]);
    }
    const double nzc = s * cs * cs;
    const double sc = (nzc < norm_Z && nzc > kNumPrecision) ? sqrt(norm_Z / nzc) : 1.0;
    const double zt = sc * fma(-gtz, dgn, sh.vp[c]);
    sh.cs[c] = cs * sc;
    sh.ztg[c] = zt;
    sh.zs[c] = zt * (cs * sc);
  }
  __syncthreads();
  return norm_Z;
}

// Search direction d = -Z Z^T g with Z = Zs diag(cs) (get_search_direction,
// BFGS_Powell.cpp:407-446); Z^T g (ztg) and cs * Z^T g (zs) come from the last update or, for
// Z = I, are g itself.  Returns d.g, the maximal step and g.g.
template <class ZA>
static __device__ void bfgs_direction(int P, const BfgsVecs& sh, double& dg, double& max_step, double& gn,
                                      const ZA& za) {
  const double* Z = sh.Z;
  for (int r = threadIdx.x; r < P; r += blockDim.x) {
    const double* row = Z + (long long)r * P;
    double s = 0.0;
#pragma unroll 8
    for (int c = 0; c < P; c++) s = fma(-za.ld(row + c), sh.zs[c], s);
    sh.d[r] = s;
  }
  __syncthreads();
  dg = dot(sh.d, sh.g, P, sh.scratch);
  max_step = 0.0;
  if (dg < 0.0) {
    // min_k |2 pi / d_k| over |d_k| >= 1e-5 (grad_descend.cpp:399-425) is 2 pi / max_k |d_k|:
    // correctly rounded division is monotone, so one division gives the same value
    double dmax = 0.0;
    for (int k = threadIdx.x; k < P; k += blockDim.x)
      if (fabs(sh.d[k]) >= 1e-5) dmax = fmax(dmax, fabs(sh.d[k]));
    dmax = -block_allmin(-dmax, sh.scratch);
    max_step = dmax > 0.0 ? kTwoPi / dmax : 0.0;
  }
  gn = dot(sh.g, sh.g, P, sh.scratch);
}

}  // namespace sqg
