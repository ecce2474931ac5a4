// Geodesic FWHM smoothing of surface images: the GB300 form of calc_gd_fwhm
// (tfce_mediation/cynumstats.pyx:76-107) as tools/tm_gd_fwhm_smoothing.py:96
// runs it on every subject image of a study.
//
// The reference walks the pair list (i, j, distance) once per image and
// scatters: sumval[j] += w * data[i], sumval[i] += w * data[j], and w into
// both weight sums, then adds every vertex's self weight and divides.  Here
// the pair list is turned once (host) into a per-vertex gather list in pair
// order -- entry (source vertex, pair index) -- so one thread owns one vertex
// of one image and adds its contributions in exactly the reference's order,
// in float32 with one rounding per product and one per sum (the reference's
// accumulators are float32 array items updated through numpy scalars).  No
// atomics, deterministic, B images per launch.
//
// Weights (gd_fwhm_weights): pdf_compute(distance, 0, scale) with the
// reference's mixed precision: norm = float(sqrt(2 pi scale)) in double,
// exponent = float(-(d*d) / (2 scale)) with d*d rounded to float and the
// division in double, weight = float((1/norm) * float(exp(exponent))).  The
// float square and exponential are correctly rounded here; the reference's
// libm powf / expf are within 1 ulp of that (they differ on ~0.06 % of
// arguments), which can move a smoothed value by an ulp.
#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace tfgb {

__device__ inline float gd_weight(float x, float scale, double inv_norm) {
  const float d = __fsub_rn(x, 0.0f);
  const float p = __fmul_rn(d, d);
  const float ex = __double2float_rn((-1.0 * static_cast<double>(p)) / (2.0 * static_cast<double>(scale)));
  const float e = __double2float_rn(exp(static_cast<double>(ex)));
  return __double2float_rn(inv_norm * static_cast<double>(e));
}

__global__ void gd_weight_kernel(const float* __restrict__ dist, int64_t M, float scale, double inv_norm,
                                 float* __restrict__ w) {
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x <= M; x += (int64_t)gridDim.x * blockDim.x)
    w[x] = gd_weight(x < M ? dist[x] : 0.0f, scale, inv_norm);  // w[M]: the self weight
}

__global__ void gd_smooth_kernel(const int64_t* __restrict__ off, const int32_t* __restrict__ src,
                                 const int32_t* __restrict__ pidx, const float* __restrict__ w, int64_t M,
                                 const float* __restrict__ data, int64_t ld, int32_t V, float* __restrict__ out,
                                 int64_t ldo, int32_t* err) {
  const int32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t b = blockIdx.y;
  if (v >= V) return;
  const float* img = data + b * ld;
  float s = 0.0f, sw = 0.0f;
  bool bad = false;
  const int64_t k1 = off[v + 1];
  for (int64_t k = off[v]; k < k1; ++k) {
    const int32_t u = src[k], x = pidx[k];
    if (static_cast<unsigned>(u) >= static_cast<unsigned>(V) || x < 0 || x >= M) {
      bad = true;
      continue;
    }
    const float wk = w[x];
    s = __fadd_rn(s, __fmul_rn(wk, img[u]));
    sw = __fadd_rn(sw, wk);
  }
  const float w0 = w[M];
  s = __fadd_rn(s, __fmul_rn(w0, img[v]));
  sw = __fadd_rn(sw, w0);
  out[b * ldo + v] = __fdiv_rn(s, sw);
  if (bad) atomicExch(err, kDevBadIndex);
}

}  // namespace tfgb

extern "C" {

int gd_fwhm_weights(const float* dist, int64_t M, float scale, float* w, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(w && (M == 0 || dist), "NULL pointer");
  TFGB_CHECK_ARG(M >= 0, "M must be >= 0");
  TFGB_CHECK_ARG(std::isfinite(scale) && scale > 0.0f, "scale must be finite and > 0");
  const float norm = static_cast<float>(std::sqrt((2.0 * M_PI) * static_cast<double>(scale)));
  const double inv_norm = 1.0 / static_cast<double>(norm);
  const unsigned blocks = static_cast<unsigned>(std::min<int64_t>((M + 256) / 256, 152 * 16));
  tfgb::gd_weight_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(dist, M, scale, inv_norm, w);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

int gd_fwhm_smooth(const int64_t* off, const int32_t* src, const int32_t* pidx, const float* w, int64_t M,
                   const float* data, int64_t ld, int32_t B, int32_t V, float* out, int64_t ldo, int32_t* err,
                   void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(off && w && data && out && err, "NULL pointer");
  TFGB_CHECK_ARG(M >= 0 && B >= 0 && V >= 0 && ld >= V && ldo >= V, "bad sizes");
  TFGB_CHECK_ARG(B <= 65535, "at most 65535 images per launch");
  if (B == 0 || V == 0) return TFCE_OK;
  const dim3 grid(static_cast<unsigned>((V + 255) / 256), static_cast<unsigned>(B));
  tfgb::gd_smooth_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(off, src, pidx, w, M, data, ld, V, out,
                                                                              ldo, err);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

}  // extern "C"
