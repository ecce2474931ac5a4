// Small-MLP training and inference kernels for the learned null-tail
// surrogate (the reference has no counterpart; its precedent is the gamma /
// Johnson-SB tail fits of bin/tm_maths:522-553).
//
// mlp_gemm:       C = op(A) . op(B) (+ bias) (+ C if accumulate), optional GELU
//                 epilogue that also stores the pre-activation (FP32);
// mlp_gemm_bf16:  the same forward GEMM with bfloat16 A and B (inference),
//                 FP32 accumulation;
// mlp_gelu_backward, mlp_bias_grad, mlp_mse_loss, mlp_adam_step: the rest of
// a training step.
// GEMM tiles are 64 x 64 outputs per 256-thread CTA, 16-deep K slices staged
// in shared memory, 4 x 4 outputs per thread.
#include <cuda_bf16.h>

#include "common.cuh"

namespace tfgb {

constexpr int kMT = 64, kNT = 64, kKT = 16;

__device__ inline float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }

__device__ inline float gelu_grad(float x) {
  const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * __expf(-0.5f * x * x);
  return cdf + x * pdf;
}

template <typename T>
__device__ inline float to_f(T v);
template <>
__device__ inline float to_f<float>(float v) { return v; }
template <>
__device__ inline float to_f<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

// element (r, c) of op(X) where X is stored row-major with leading dimension ld
template <typename T>
__device__ inline float at(const T* X, int ld, bool trans, int r, int c) {
  return trans ? to_f<T>(X[(int64_t)c * ld + r]) : to_f<T>(X[(int64_t)r * ld + c]);
}

template <typename T>
__global__ void __launch_bounds__(256) gemm_kernel(int transA, int transB, int M, int N, int K,
                                                   const T* __restrict__ A, int lda,
                                                   const T* __restrict__ B, int ldb,
                                                   float* __restrict__ C, int ldc,
                                                   const float* __restrict__ bias, int act,
                                                   float* __restrict__ preact, int accumulate) {
  __shared__ float sA[kKT][kMT + 1];
  __shared__ float sB[kKT][kNT + 1];
  const int m0 = blockIdx.y * kMT, n0 = blockIdx.x * kNT;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += kKT) {
    for (int i = threadIdx.x; i < kKT * kMT; i += 256) {
      const int kk = i / kMT, mm = i % kMT;
      const int r = m0 + mm, c = k0 + kk;
      sA[kk][mm] = (r < M && c < K) ? at<T>(A, lda, transA, r, c) : 0.0f;
    }
    for (int i = threadIdx.x; i < kKT * kNT; i += 256) {
      const int kk = i / kNT, nn = i % kNT;
      const int r = k0 + kk, c = n0 + nn;
      sB[kk][nn] = (r < K && c < N) ? at<T>(B, ldb, transB, r, c) : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kKT; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = sA[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = sB[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = m0 + ty * 4 + i;
    if (r >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = n0 + tx * 4 + j;
      if (c >= N) continue;
      float v = acc[i][j];
      if (bias) v += bias[c];
      if (accumulate) v += C[(int64_t)r * ldc + c];
      if (preact) preact[(int64_t)r * ldc + c] = v;
      if (act == 1) v = gelu(v);
      C[(int64_t)r * ldc + c] = v;
    }
  }
}

__global__ void gelu_backward_kernel(const float* __restrict__ dy, const float* __restrict__ z,
                                     float* __restrict__ dz, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dz[i] = dy[i] * gelu_grad(z[i]);
}

// db[c] = sum over rows of dz[r][c] (deterministic: one thread per column)
__global__ void bias_grad_kernel(const float* __restrict__ dz, int rows, int cols, float* __restrict__ db) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.0f;
  for (int r = 0; r < rows; ++r) s += dz[(int64_t)r * cols + c];
  db[c] = s;
}

// loss = mean((y - t)^2 * w) over n entries; dy = 2 (y - t) w / n.  One CTA.
__global__ void mse_kernel(const float* __restrict__ y, const float* __restrict__ t,
                           const float* __restrict__ w, int64_t n, int cols, float* __restrict__ dy,
                           float* __restrict__ loss) {
  __shared__ float red[256];
  float s = 0.0f;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const float wi = w ? w[i % cols] : 1.0f;
    const float d = y[i] - t[i];
    s += d * d * wi;
    dy[i] = 2.0f * d * wi / static_cast<float>(n);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = red[0] / static_cast<float>(n);
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps,
                            float bc1, float bc2, float wd) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i] + wd * p[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  }
}

__global__ void to_bf16_kernel(const float* __restrict__ x, __nv_bfloat16* __restrict__ y, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16_rn(x[i]);
}

inline unsigned grid1d(int64_t n) { return static_cast<unsigned>(std::min<int64_t>((n + 255) / 256, 2048)); }

}  // namespace tfgb

extern "C" {

int mlp_gemm(int32_t transA, int32_t transB, int32_t M, int32_t N, int32_t K, const float* A, int32_t lda,
             const float* B, int32_t ldb, float* C, int32_t ldc, const float* bias, int32_t act,
             float* preact, int32_t accumulate, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(A && B && C, "NULL pointer");
  TFGB_CHECK_ARG(M >= 0 && N >= 0 && K >= 0, "bad sizes");
  TFGB_CHECK_ARG(act == 0 || act == 1, "act must be 0 (none) or 1 (GELU)");
  if (M == 0 || N == 0) return TFCE_OK;
  dim3 grid((N + tfgb::kNT - 1) / tfgb::kNT, (M + tfgb::kMT - 1) / tfgb::kMT);
  tfgb::gemm_kernel<float><<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      transA, transB, M, N, K, A, lda, B, ldb, C, ldc, bias, act, preact, accumulate);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

int mlp_gemm_bf16(int32_t transA, int32_t transB, int32_t M, int32_t N, int32_t K, const void* A, int32_t lda,
                  const void* B, int32_t ldb, float* C, int32_t ldc, const float* bias, int32_t act,
                  void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(A && B && C, "NULL pointer");
  TFGB_CHECK_ARG(M >= 0 && N >= 0 && K >= 0, "bad sizes");
  TFGB_CHECK_ARG(act == 0 || act == 1, "act must be 0 (none) or 1 (GELU)");
  if (M == 0 || N == 0) return TFCE_OK;
  dim3 grid((N + tfgb::kNT - 1) / tfgb::kNT, (M + tfgb::kMT - 1) / tfgb::kMT);
  tfgb::gemm_kernel<__nv_bfloat16><<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      transA, transB, M, N, K, static_cast<const __nv_bfloat16*>(A), lda, static_cast<const __nv_bfloat16*>(B),
      ldb, C, ldc, bias, act, nullptr, 0);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

int mlp_to_bf16(const float* x, void* y, int64_t n, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(x && y && n >= 0, "bad arguments");
  if (n == 0) return TFCE_OK;
  tfgb::to_bf16_kernel<<<tfgb::grid1d(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      x, static_cast<__nv_bfloat16*>(y), n);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

int mlp_gelu_backward(const float* dy, const float* z, float* dz, int64_t n, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(dy && z && dz && n >= 0, "bad arguments");
  if (n == 0) return TFCE_OK;
  tfgb::gelu_backward_kernel<<<tfgb::grid1d(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(dy, z, dz, n);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

int mlp_bias_grad(const float* dz, int32_t rows, int32_t cols, float* db, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(dz && db && rows >= 0 && cols >= 0, "bad arguments");
  if (cols == 0) return TFCE_OK;
  tfgb::bias_grad_kernel<<<(cols + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(dz, rows, cols, db);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

int mlp_mse_loss(const float* y, const float* t, const float* col_weight, int64_t n, int32_t cols, float* dy,
                 float* loss, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(y && t && dy && loss && n >= 1 && cols >= 1, "bad arguments");
  tfgb::mse_kernel<<<1, 256, 0, static_cast<cudaStream_t>(stream)>>>(y, t, col_weight, n, cols, dy, loss);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

int mlp_adam_step(float* param, const float* grad, float* m, float* v, int64_t n, float lr, float beta1,
                  float beta2, float eps, int32_t step, float weight_decay, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(param && grad && m && v && n >= 0 && step >= 1, "bad arguments");
  if (n == 0) return TFCE_OK;
  const float bc1 = 1.0f - powf(beta1, static_cast<float>(step));
  const float bc2 = 1.0f - powf(beta2, static_cast<float>(step));
  tfgb::adam_kernel<<<tfgb::grid1d(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      param, grad, m, v, n, lr, beta1, beta2, eps, bc1, bc2, weight_decay);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

}  // extern "C"
