// Mass-univariate OLS t-statistics for many designs against one data matrix:
// the GB300 replacement of tval_int / se_of_slope / calc_beta_se
// (tfce_mediation/cynumstats.pyx:28-29, 47-74) and of the per-permutation
// design loop of tfce_mediation/tmanalysis/vertex_tfce_multiple_regression_randomise.py:90-107.
//
// One CTA owns a tile of kTileV vertex columns of Y (all n subjects, held in
// shared memory) and runs every design of the batch over it, so Y is read
// from HBM once per batch.  For design g and column v:
//   beta_j = sum_s pinv[g][j][s] * y[s][v]                (cy_lin_lstsqr_mat)
//   rss    = sum_s (y[s][v] - sum_j X[g][s][j] beta_j)^2  (residuals, never Y'Y)
//   t_j    = beta_j / sqrt(rss / dof_g * invdiag[g][j])   (se_of_slope, tval_int)
// in FP32 with FMA accumulation; the FP64 k x k inverse and pseudoinverse are
// formed on the host.
//
// Also: the indirect-effect (Sobel/Aroian/Goodman) combination of two path t
// maps (tfce_mediation/pyfunc.py:146-161).
#include <algorithm>

#include <math_constants.h>

#include "common.cuh"

namespace tfgb {

constexpr int kGlmThreads = 256;
constexpr int kColsPerThread = 4;

// Y tile [n][TV] in shared memory; each thread computes 4 adjacent columns of
// one design; TV/4 threads per design; kGlmThreads/(TV/4) designs in flight.
enum GlmWhat : int32_t { kWhatT = 0, kWhatBeta = 1, kWhatSE = 2, kWhatResid = 3, kWhatF = 4, kWhatRSS = 5 };

template <int KMAX, int TV>
__global__ void __launch_bounds__(kGlmThreads) glm_tstat_kernel(
    const float* __restrict__ Y, int64_t ldy, int32_t n, int64_t V,
    const float* __restrict__ pinv, const float* __restrict__ X,
    const float* __restrict__ invdiag, const float* __restrict__ dof, int32_t G,
    const int32_t* __restrict__ coef, int32_t n_coef, float* __restrict__ t_out, int64_t ldt,
    int32_t what) {
  extern __shared__ float4 smem4[];
  float* ys = reinterpret_cast<float*>(smem4);
  constexpr int kThreadsPerDesign = TV / kColsPerThread;
  constexpr int kDesignsInFlight = kGlmThreads / kThreadsPerDesign;
  const int64_t vbase = (int64_t)blockIdx.x * TV;

  // stage the tile (zero-filled past V)
  for (int i = threadIdx.x; i < n * TV; i += kGlmThreads) {
    const int s = i / TV, c = i % TV;
    const int64_t v = vbase + c;
    ys[i] = (v < V) ? Y[(int64_t)s * ldy + v] : 0.0f;
  }
  __syncthreads();

  const int lane_d = threadIdx.x % kThreadsPerDesign;
  const int slot = threadIdx.x / kThreadsPerDesign;
  const int c0 = lane_d * kColsPerThread;
  const float4* yrow = reinterpret_cast<const float4*>(ys) + lane_d;  // stride TV/4 per subject

  for (int g = slot; g < G; g += kDesignsInFlight) {
    const float* pg = pinv + (int64_t)g * KMAX * n;
    const float* xg = X + (int64_t)g * n * KMAX;
    float b[KMAX][kColsPerThread];
#pragma unroll
    for (int j = 0; j < KMAX; ++j)
#pragma unroll
      for (int c = 0; c < kColsPerThread; ++c) b[j][c] = 0.0f;
    for (int s = 0; s < n; ++s) {
      const float4 y = yrow[s * (TV / 4)];
#pragma unroll
      for (int j = 0; j < KMAX; ++j) {
        const float w = __ldg(pg + (int64_t)j * n + s);
        b[j][0] = fmaf(w, y.x, b[j][0]);
        b[j][1] = fmaf(w, y.y, b[j][1]);
        b[j][2] = fmaf(w, y.z, b[j][2]);
        b[j][3] = fmaf(w, y.w, b[j][3]);
      }
    }
    float rss[kColsPerThread] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int s = 0; s < n; ++s) {
      const float4 y = yrow[s * (TV / 4)];
      float r0 = y.x, r1 = y.y, r2 = y.z, r3 = y.w;
#pragma unroll
      for (int j = 0; j < KMAX; ++j) {
        const float xv = __ldg(xg + (int64_t)s * KMAX + j);
        r0 = fmaf(-xv, b[j][0], r0);
        r1 = fmaf(-xv, b[j][1], r1);
        r2 = fmaf(-xv, b[j][2], r2);
        r3 = fmaf(-xv, b[j][3], r3);
      }
      rss[0] = fmaf(r0, r0, rss[0]);
      rss[1] = fmaf(r1, r1, rss[1]);
      rss[2] = fmaf(r2, r2, rss[2]);
      rss[3] = fmaf(r3, r3, rss[3]);
      if (what == kWhatResid) {
        float* dst = t_out + ((int64_t)g * n + s) * ldt + vbase + c0;
        const float rr[4] = {r0, r1, r2, r3};
#pragma unroll
        for (int c = 0; c < kColsPerThread; ++c)
          if (vbase + c0 + c < V) dst[c] = rr[c];
      }
    }
    if (what == kWhatResid) continue;
    if (what == kWhatRSS || what == kWhatF) {
      float outv[kColsPerThread];
      if (what == kWhatRSS) {
#pragma unroll
        for (int c = 0; c < kColsPerThread; ++c) outv[c] = rss[c];
      } else {
        // F = ((TSS - RSS)/(k-1)) / (RSS/(n-k))   (cynumstats.pyx:31-36).
        // TSS is taken around a supplied centre (the reference uses the grand
        // mean of the whole matrix, np.mean(y)) passed in invdiag[0], or
        // around each column's mean when invdiag is NULL.
        float mean[kColsPerThread] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (invdiag) {
#pragma unroll
          for (int c = 0; c < kColsPerThread; ++c) mean[c] = invdiag[0];
        } else {
          for (int s = 0; s < n; ++s) {
            const float4 y = yrow[s * (TV / 4)];
            mean[0] += y.x; mean[1] += y.y; mean[2] += y.z; mean[3] += y.w;
          }
          const float inv_n = 1.0f / static_cast<float>(n);
#pragma unroll
          for (int c = 0; c < kColsPerThread; ++c) mean[c] *= inv_n;
        }
        float tss[kColsPerThread] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (int s = 0; s < n; ++s) {
          const float4 y = yrow[s * (TV / 4)];
          const float d0 = y.x - mean[0], d1 = y.y - mean[1], d2 = y.z - mean[2], d3 = y.w - mean[3];
          tss[0] = fmaf(d0, d0, tss[0]); tss[1] = fmaf(d1, d1, tss[1]);
          tss[2] = fmaf(d2, d2, tss[2]); tss[3] = fmaf(d3, d3, tss[3]);
        }
        const float dg = dof[g];
        const float km1 = static_cast<float>(n) - dg - 1.0f;
#pragma unroll
        for (int c = 0; c < kColsPerThread; ++c) outv[c] = ((tss[c] - rss[c]) / km1) / (rss[c] / dg);
      }
      float* dst = t_out + (int64_t)g * ldt + vbase + c0;
#pragma unroll
      for (int c = 0; c < kColsPerThread; ++c)
        if (vbase + c0 + c < V) dst[c] = outv[c];
      continue;
    }
    const float inv_dof = 1.0f / dof[g];
    for (int ci = 0; ci < n_coef; ++ci) {
      const int j = coef[ci];
      const float d = invdiag[(int64_t)g * KMAX + j];
      float* dst = t_out + ((int64_t)g * n_coef + ci) * ldt + vbase + c0;
#pragma unroll
      for (int c = 0; c < kColsPerThread; ++c) {
        if (vbase + c0 + c < V) {
          float bj = 0.0f;
#pragma unroll
          for (int jj = 0; jj < KMAX; ++jj)
            if (jj == j) bj = b[jj][c];
          const float se = sqrtf(rss[c] * inv_dof * d);
          dst[c] = (what == kWhatT) ? bj / se : (what == kWhatBeta) ? bj : se;
        }
      }
    }
  }
}

template <int KMAX>
int launch_glm_k(int tv, const float* Y, int64_t ldy, int32_t n, int64_t V, const float* pinv,
                 const float* X, const float* invdiag, const float* dof, int32_t G,
                 const int32_t* coef, int32_t n_coef, float* t_out, int64_t ldt, int32_t what,
                 cudaStream_t st) {
  const size_t smem = sizeof(float) * (size_t)n * tv;
  const unsigned grid = static_cast<unsigned>((V + tv - 1) / tv);
#define TFGB_GLM_LAUNCH(TVV)                                                                   \
  do {                                                                                         \
    auto kern = glm_tstat_kernel<KMAX, TVV>;                                                   \
    TFGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,         \
                                   static_cast<int>(smem)));                                   \
    kern<<<grid, kGlmThreads, smem, st>>>(Y, ldy, n, V, pinv, X, invdiag, dof, G, coef,        \
                                          n_coef, t_out, ldt, what);                           \
  } while (0)
  if (tv == 64) TFGB_GLM_LAUNCH(64);
  else if (tv == 32) TFGB_GLM_LAUNCH(32);
  else TFGB_GLM_LAUNCH(16);
#undef TFGB_GLM_LAUNCH
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

// FP64 form for the observed (unpermuted) statistic and the one-off helpers,
// with the reference's precision: betas and sigma^2 in double from the float32
// data, the SE rounded to float32 (se_of_slope stores it in a float32 array,
// cynumstats.pyx:47-52) and t = double beta / that SE (tval_int, :59-64).
// One thread per vertex, the design's pseudoinverse and rows in shared memory.
template <int KMAX>
__global__ void __launch_bounds__(256) glm_f64_kernel(
    const float* __restrict__ Y, int64_t ldy, int32_t n, int64_t V, const double* __restrict__ pinv,
    const double* __restrict__ X, const double* __restrict__ invdiag, const double* __restrict__ dof,
    const int32_t* __restrict__ coef, int32_t n_coef, int32_t what, double* __restrict__ out, int64_t ldo) {
  extern __shared__ double sm64[];
  double* ps = sm64;              // [KMAX][n]
  double* xs = sm64 + KMAX * n;   // [n][KMAX]
  const int64_t g = blockIdx.y;
  for (int i = threadIdx.x; i < KMAX * n; i += blockDim.x) {
    ps[i] = pinv[g * KMAX * n + i];
    xs[i] = X[g * n * KMAX + i];
  }
  __syncthreads();
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V) return;
  double b[KMAX];
#pragma unroll
  for (int j = 0; j < KMAX; ++j) b[j] = 0.0;
  for (int s = 0; s < n; ++s) {
    const double y = (double)Y[(int64_t)s * ldy + v];
#pragma unroll
    for (int j = 0; j < KMAX; ++j) b[j] = fma(ps[j * n + s], y, b[j]);
  }
  double rss = 0.0;
  for (int s = 0; s < n; ++s) {
    double r = (double)Y[(int64_t)s * ldy + v];
#pragma unroll
    for (int j = 0; j < KMAX; ++j) r = fma(-xs[s * KMAX + j], b[j], r);
    rss = fma(r, r, rss);
  }
  const double sigma2 = rss / dof[g];
  for (int c = 0; c < n_coef; ++c) {
    const int j = coef[c];
    double bj = 0.0;
#pragma unroll
    for (int jj = 0; jj < KMAX; ++jj)
      if (jj == j) bj = b[jj];
    double* dst = out + (g * n_coef + c) * ldo + v;
    if (j < 0 || j >= KMAX) {
      *dst = CUDART_NAN;
      continue;
    }
    const double se = (double)__double2float_rn(sqrt(sigma2 * invdiag[g * KMAX + j]));
    *dst = (what == kWhatBeta) ? bj : (what == kWhatSE) ? se : bj / se;
  }
}

// Aroian (0), Sobel (1), Goodman (2) z from path t values, in double like
// the reference's numpy expression, stored as float32.
__global__ void sobel_combine_kernel(const float* __restrict__ ta, int64_t lda,
                                     const float* __restrict__ ta_scalar,
                                     const float* __restrict__ tb, int64_t ldb, int32_t P,
                                     int64_t V, int32_t alg, float* __restrict__ z, int64_t ldz) {
  const int64_t total = (int64_t)P * V;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = i / V, v = i % V;
    const double a = ta ? (double)ta[p * lda + v] : (double)ta_scalar[p];
    const double b = (double)tb[p * ldb + v];
    const double ia = 1.0 / (a * a), ib = 1.0 / (b * b), iab = 1.0 / (a * a * b * b);
    double q;
    if (alg == 0) q = ib + ia + iab;
    else if (alg == 1) q = ib + ia;
    else q = ib + ia - iab;
    z[p * ldz + v] = (float)(1.0 / sqrt(q));
  }
}

}  // namespace tfgb

extern "C" {

int glm_stat(const float* Y, int64_t ldy, int32_t n, int64_t V, const float* pinv, const float* X,
             const float* invdiag, const float* dof, int32_t G, int32_t kmax, const int32_t* coef,
             int32_t n_coef, int32_t what, float* out, int64_t ldo, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(Y && pinv && X && dof && out, "NULL pointer");
  TFGB_CHECK_ARG(what >= 0 && what <= 5, "what must be in [0, 5]");
  const bool per_coef = (what <= 2);
  TFGB_CHECK_ARG(!per_coef || (coef && n_coef >= 1), "coef list required");
  TFGB_CHECK_ARG(what == 1 || what == 3 || what == 4 || what == 5 || invdiag, "invdiag is NULL");
  if (what != 4 && what != 0 && what != 2) invdiag = nullptr;  // unused
  TFGB_CHECK_ARG(n > 0 && V >= 0 && G >= 0, "bad sizes");
  TFGB_CHECK_ARG(kmax >= 1 && kmax <= 8, "kmax must be in [1, 8]");
  TFGB_CHECK_ARG(ldy >= V && ldo >= V, "leading dimension < V");
  if (V == 0 || G == 0) return TFCE_OK;
  int tv;
  if ((size_t)n * 64 * 4 <= 200 * 1024) tv = 64;
  else if ((size_t)n * 32 * 4 <= 200 * 1024) tv = 32;
  else if ((size_t)n * 16 * 4 <= 200 * 1024) tv = 16;
  else {
    tfgb::set_error("n = %d subjects exceeds the shared-memory tile (max 3200)", n);
    return TFCE_EINVAL;
  }
  if (!per_coef) {
    coef = nullptr;
    n_coef = 0;
  }
  const float* idg = invdiag;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  switch (kmax) {
#define TFGB_K(KK) \
    case KK: return tfgb::launch_glm_k<KK>(tv, Y, ldy, n, V, pinv, X, idg, dof, G, coef, n_coef, out, ldo, what, st);
    TFGB_K(1) TFGB_K(2) TFGB_K(3) TFGB_K(4) TFGB_K(5) TFGB_K(6) TFGB_K(7)
    default: return tfgb::launch_glm_k<8>(tv, Y, ldy, n, V, pinv, X, idg, dof, G, coef, n_coef, out, ldo, what, st);
#undef TFGB_K
  }
}

int glm_tstat(const float* Y, int64_t ldy, int32_t n, int64_t V, const float* pinv, const float* X,
              const float* invdiag, const float* dof, int32_t G, int32_t kmax,
              const int32_t* coef, int32_t n_coef, float* t_out, int64_t ldt, void* stream) {
  return glm_stat(Y, ldy, n, V, pinv, X, invdiag, dof, G, kmax, coef, n_coef, 0, t_out, ldt, stream);
}

int glm_fstat(const float* Y, int64_t ldy, int32_t n, int64_t V, const float* pinv, const float* X,
              const float* dof, int32_t G, int32_t kmax, const float* centre, float* f_out,
              int64_t ldf, void* stream) {
  return glm_stat(Y, ldy, n, V, pinv, X, centre, dof, G, kmax, nullptr, 0, 4, f_out, ldf, stream);
}

int glm_stat_f64(const float* Y, int64_t ldy, int32_t n, int64_t V, const double* pinv, const double* X,
                 const double* invdiag, const double* dof, int32_t G, int32_t kmax, const int32_t* coef,
                 int32_t n_coef, int32_t what, double* out, int64_t ldo, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(Y && pinv && X && dof && out && coef, "NULL pointer");
  TFGB_CHECK_ARG(what >= 0 && what <= 2, "what must be 0 (t), 1 (beta) or 2 (se)");
  TFGB_CHECK_ARG(what == 1 || invdiag, "invdiag is NULL");
  TFGB_CHECK_ARG(n > 0 && V >= 0 && G >= 0 && n_coef >= 1, "bad sizes");
  TFGB_CHECK_ARG(kmax >= 1 && kmax <= 8, "kmax must be in [1, 8]");
  TFGB_CHECK_ARG(ldy >= V && ldo >= V, "leading dimension < V");
  TFGB_CHECK_ARG(G < 65536, "at most 65535 designs per launch");
  const size_t smem = sizeof(double) * 2 * (size_t)kmax * n;
  if (smem > 200 * 1024) {
    tfgb::set_error("n = %d subjects x %d columns exceeds the shared-memory design tile", n, kmax);
    return TFCE_EINVAL;
  }
  if (V == 0 || G == 0) return TFCE_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const dim3 grid(static_cast<unsigned>((V + 255) / 256), static_cast<unsigned>(G));
  switch (kmax) {
#define TFGB_K64(KK)                                                                                   \
    case KK: {                                                                                         \
      const size_t sm = sizeof(double) * 2 * KK * (size_t)n;                                           \
      TFGB_CUDA(cudaFuncSetAttribute(tfgb::glm_f64_kernel<KK>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                     static_cast<int>(sm)));                                           \
      tfgb::glm_f64_kernel<KK><<<grid, 256, sm, st>>>(Y, ldy, n, V, pinv, X, invdiag, dof, coef, n_coef, \
                                                      what, out, ldo);                                 \
      break;                                                                                           \
    }
    TFGB_K64(1) TFGB_K64(2) TFGB_K64(3) TFGB_K64(4) TFGB_K64(5) TFGB_K64(6) TFGB_K64(7) TFGB_K64(8)
#undef TFGB_K64
    default: break;
  }
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

int sobel_combine(const float* ta, int64_t lda, const float* ta_scalar, const float* tb,
                  int64_t ldb, int32_t P, int64_t V, int32_t alg, float* z, int64_t ldz,
                  void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG((ta || ta_scalar) && tb && z, "NULL pointer");
  TFGB_CHECK_ARG(alg >= 0 && alg <= 2, "alg must be 0 (aroian), 1 (sobel) or 2 (goodman)");
  TFGB_CHECK_ARG(P >= 0 && V >= 0, "bad sizes");
  if (P == 0 || V == 0) return TFCE_OK;
  const int64_t total = (int64_t)P * V;
  const int threads = 256;
  const unsigned blocks = static_cast<unsigned>(std::min<int64_t>((total + threads - 1) / threads, 152 * 32));
  tfgb::sobel_combine_kernel<<<blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(
      ta, lda, ta_scalar, tb, ldb, P, V, alg, z, ldz);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

}  // extern "C"
