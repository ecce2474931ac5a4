// FWER lookups: sort the permutation maxima and map TFCE images to 1-p(FWER),
// the GB300 replacement of
//   tfce_mediation/tmanalysis/calculate_fweP_vertex.py:37-69 (mode 0),
//   tfce_mediation/tmanalysis/calculate_fweP_voxel.py:23-49   (mode 0),
//   tfce_mediation/tm_func.py:566-573 / pyfunc.py:254-261      (mode 1).
// The sort is a bitonic network in its "mirror first" form: every
// compare-exchange puts the smaller value at the lower index, so lengths that
// are not a power of two are handled by treating missing elements as +inf
// without storing them (no scratch buffer).
#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace tfgb {

__global__ void bitonic_step(double* __restrict__ a, int64_t n, int64_t half_pairs, int64_t j,
                             int mirror) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < half_pairs;
       t += (int64_t)gridDim.x * blockDim.x) {
    // t enumerates the lower elements of the pairs: insert a zero bit at j
    const int64_t i = ((t / j) * 2 * j) + (t % j);
    const int64_t l = mirror ? (i ^ (2 * j - 1)) : (i + j);
    if (l >= n) continue;  // partner is padding (+inf): already in order
    const double x = a[i], y = a[l];
    if (y < x) {
      a[i] = y;
      a[l] = x;
    }
  }
}

__device__ inline int64_t lower_bound(const double* a, int64_t n, double x) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__global__ void fwer_lookup_kernel(const double* __restrict__ srt, int64_t N,
                                   const double* __restrict__ img, int64_t V, int mode,
                                   double* __restrict__ out) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V;
       v += (int64_t)gridDim.x * blockDim.x) {
    const double x = img[v];
    double p = 0.0;
    if (mode == 0) {
      if (x > 0.0) {
        const int64_t idx = lower_bound(srt, N, x);
        p = (idx == 0) ? 0.0 : (double)(idx - 1) / (double)N;
      }
    } else {
      const int64_t idx = lower_bound(srt, N, x);
      if (idx == N) {
        p = (double)(N - 1) / (double)N;
      } else {
        // idx - 1 == -1 wraps to the last element, as numpy indexing does
        const int64_t lo = (idx == 0) ? N - 1 : idx - 1;
        if (fabs(x - srt[lo]) < fabs(x - srt[idx])) p = (double)lo / (double)N;
        else p = (double)idx / (double)N;
      }
    }
    out[v] = p;
  }
}

}  // namespace tfgb

extern "C" {

int fwer_sort(double* values, int64_t n, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(n >= 0, "n < 0");
  TFGB_CHECK_ARG(n == 0 || values != nullptr, "values is NULL");
  if (n < 2) return TFCE_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int64_t n2 = 1;
  while (n2 < n) n2 <<= 1;
  const int64_t pairs = n2 / 2;
  const int threads = 256;
  const unsigned blocks = static_cast<unsigned>(std::min<int64_t>((pairs + threads - 1) / threads, 4096));
  for (int64_t k = 2; k <= n2; k <<= 1) {
    tfgb::bitonic_step<<<blocks, threads, 0, st>>>(values, n, pairs, k / 2, 1);
    for (int64_t j = k / 4; j >= 1; j >>= 1)
      tfgb::bitonic_step<<<blocks, threads, 0, st>>>(values, n, pairs, j, 0);
  }
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

int fwer_lookup(const double* sorted_null, int64_t N, const double* image, int64_t V, int32_t mode,
                double* out, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(N >= 1, "empty null distribution");
  TFGB_CHECK_ARG(sorted_null && image && out, "NULL pointer");
  TFGB_CHECK_ARG(mode == 0 || mode == 1, "mode must be 0 or 1");
  if (V <= 0) return TFCE_OK;
  const int threads = 256;
  const unsigned blocks = static_cast<unsigned>(std::min<int64_t>((V + threads - 1) / threads, 152 * 16));
  tfgb::fwer_lookup_kernel<<<blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(
      sorted_null, N, image, V, mode, out);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

}  // extern "C"
