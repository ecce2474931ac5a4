// Repeated-measures ANCOVA F maps of permuted designs: the GB300 form of the
// statistics of reg_rm_ancova_one_bs_factor / reg_rm_ancova_two_bs_factor
// (tfce_mediation/pyfunc.py:2067-2280, 1712-2060) as the tm-models
// permutation loop calls them (tmanalysis/tm_models_randomise.py:522-684).
//
// Every effect sum of squares of those functions is the extra sum of squares
// of dropping a column group S from one design; the tensor-core GLM forms them
// in Wald form (glm_stat_tc mode 4).  What is left per permutation and vertex
// is the subject split of the total sum of squares -- the fit on the subject
// dummies, i.e. the sums of squares between and within subject means -- and
// the F ratios:
//   SS_between = sum_g |g| (mean_g - mean)^2,  SS_within = sum_g sum_{i in g} (y_i - mean_g)^2
//   error_between = SS_between - sum of its ESS rows (the between-subject cells)
//   error_within  = SS_within  - sum of its ESS rows (time and its interactions)
//   F_f = (ESS_f / df_f) / (error_f / df_error_f)
// The permuted data rows enter as an index list per permutation, grouped by
// subject: row rows[p][k] of the resident (centred) data for k in the group's
// range [goff[g], goff[g+1]).
//
// One CTA stages a 32-vertex column tile of the data (all N rows) in shared
// memory once and runs kRmPermsPerBlock permutations over it (one warp per
// permutation at a time, lane = vertex), so the data is read from HBM
// P / kRmPermsPerBlock times per batch.  A row index outside [0, N), or a
// group bound outside [0, N], is recorded in *err and clamped (the row reads
// as 0).
#include <algorithm>

#include "common.cuh"

namespace tfgb {

constexpr int kRmThreads = 256;
constexpr int kRmTile = 32;
constexpr int kRmPermsPerBlock = 64;
constexpr int kRmMaxRows = 16;
constexpr int kRmMaxF = 8;
constexpr int kRmMaxN = 1792;  // N * 32 floats of shared memory <= 224 KB

struct RmTable {
  int64_t row_off[kRmMaxRows];      // ESS row r of permutation p at ess[row_off[r] + p * row_pstride[r] + v]
  int64_t row_pstride[kRmMaxRows];
  int32_t eb_rows[kRmMaxRows];      // rows subtracted from SS_between
  int32_t ew_rows[kRmMaxRows];      // rows subtracted from SS_within
  int32_t f_num[kRmMaxF];           // numerator row of each F
  int32_t f_err[kRmMaxF];           // 0: between-subject error, 1: within-subject error
  float f_df[kRmMaxF];
  float df_b, df_w;
  int32_t n_eb, n_ew, n_f;
};

__global__ void __launch_bounds__(kRmThreads) rm_anova_kernel(const float* __restrict__ Y, int64_t ldy, int32_t N,
                                                             int64_t V, const int32_t* __restrict__ rows, int32_t P,
                                                             const int32_t* __restrict__ goff, int32_t n_groups,
                                                             const float* __restrict__ ess, RmTable tb,
                                                             float* __restrict__ out, int64_t ldo,
                                                             float* __restrict__ ss_out, int32_t* err) {
  extern __shared__ float tile[];  // [N][32]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t v0 = (int64_t)blockIdx.x * kRmTile;
  const int64_t v = v0 + lane;
  for (int e = threadIdx.x; e < N * kRmTile; e += kRmThreads) {
    const int i = e / kRmTile, l = e % kRmTile;
    tile[e] = (v0 + l < V) ? Y[(int64_t)i * ldy + v0 + l] : 0.0f;
  }
  __syncthreads();
  float tot = 0.0f;
  for (int i = 0; i < N; ++i) tot += tile[i * kRmTile + lane];
  const float mean = tot / static_cast<float>(N);
  const int p_end = min(P, (int)(blockIdx.y + 1) * kRmPermsPerBlock);
  for (int p = blockIdx.y * kRmPermsPerBlock + warp; p < p_end; p += kRmThreads / 32) {
    const int32_t* rp = rows + (int64_t)p * N;
    float ws = 0.0f, bs = 0.0f, ws_blk = 0.0f, bs_blk = 0.0f;  // two-level sums over the groups
    bool bad = false;
    for (int g = 0; g < n_groups; ++g) {
      // group bounds clamped into [0, N]: a bad table reads no row out of range
      const int g0 = __ldg(goff + g), g1 = __ldg(goff + g + 1);
      const int k0 = min(max(g0, 0), N), k1 = min(max(g1, k0), N);
      bad |= (k0 != g0) || (k1 != g1);
      float sum = 0.0f;
      for (int k = k0; k < k1; ++k) {
        const int r = __ldg(rp + k);
        const bool ok = static_cast<unsigned>(r) < static_cast<unsigned>(N);
        bad |= !ok;
        sum += ok ? tile[r * kRmTile + lane] : 0.0f;
      }
      const float cnt = static_cast<float>(k1 - k0);
      const float m = sum / cnt;
      float w = 0.0f;
      for (int k = k0; k < k1; ++k) {
        const int r = __ldg(rp + k);
        const float d = (static_cast<unsigned>(r) < static_cast<unsigned>(N) ? tile[r * kRmTile + lane] : 0.0f) - m;
        w = fmaf(d, d, w);
      }
      const float dm = m - mean;
      ws_blk += w;
      bs_blk = fmaf(cnt * dm, dm, bs_blk);
      if ((g & 15) == 15) {
        ws += ws_blk;
        bs += bs_blk;
        ws_blk = bs_blk = 0.0f;
      }
    }
    ws += ws_blk;
    bs += bs_blk;
    if (bad && lane == 0) atomicExch(err, kDevBadIndex);
    if (v >= V) continue;
    float eb = bs, ew = ws;
    for (int i = 0; i < tb.n_eb; ++i) {
      const int r = tb.eb_rows[i];
      eb -= __ldg(ess + tb.row_off[r] + (int64_t)p * tb.row_pstride[r] + v);
    }
    for (int i = 0; i < tb.n_ew; ++i) {
      const int r = tb.ew_rows[i];
      ew -= __ldg(ess + tb.row_off[r] + (int64_t)p * tb.row_pstride[r] + v);
    }
    const float msb = eb / tb.df_b, msw = ew / tb.df_w;
    for (int f = 0; f < tb.n_f; ++f) {
      const int r = tb.f_num[f];
      const float num = __ldg(ess + tb.row_off[r] + (int64_t)p * tb.row_pstride[r] + v) / tb.f_df[f];
      out[((int64_t)p * tb.n_f + f) * ldo + v] = num / (tb.f_err[f] ? msw : msb);
    }
    if (ss_out != nullptr) {
      ss_out[((int64_t)p * 2 + 0) * ldo + v] = bs;
      ss_out[((int64_t)p * 2 + 1) * ldo + v] = ws;
    }
  }
}

}  // namespace tfgb

extern "C" {

int rm_anova_max_rows(void) { return tfgb::kRmMaxN; }

int rm_anova_combine(const float* Y, int64_t ldy, int32_t N, int64_t V, const int32_t* rows, int32_t P,
                     const int32_t* goff, int32_t n_groups, const float* ess, const int64_t* row_off,
                     const int64_t* row_pstride, int32_t n_rows, const int32_t* eb_rows, int32_t n_eb,
                     const int32_t* ew_rows, int32_t n_ew, float df_b, float df_w, const int32_t* f_num,
                     const int32_t* f_err, const float* f_df, int32_t n_f, float* out, int64_t ldo, float* ss_out,
                     int32_t* err, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(Y && rows && goff && out && err, "NULL pointer");
  TFGB_CHECK_ARG(N >= 2 && N <= tfgb::kRmMaxN, "N (data rows) must be in [2, 1792]");
  TFGB_CHECK_ARG(V >= 0 && P >= 0 && ldy >= V && ldo >= V, "bad sizes");
  TFGB_CHECK_ARG(n_groups >= 1 && n_groups <= N, "n_groups must be in [1, N]");
  TFGB_CHECK_ARG(n_rows >= 0 && n_rows <= tfgb::kRmMaxRows, "at most 16 sums-of-squares rows");
  TFGB_CHECK_ARG(n_rows == 0 || (ess && row_off && row_pstride), "ESS rows need ess / row_off / row_pstride");
  TFGB_CHECK_ARG(n_eb >= 0 && n_eb <= n_rows && n_ew >= 0 && n_ew <= n_rows, "bad error-term row counts");
  TFGB_CHECK_ARG(n_f >= 0 && n_f <= tfgb::kRmMaxF, "at most 8 F maps");
  TFGB_CHECK_ARG(n_f == 0 || (f_num && f_err && f_df), "F maps need f_num / f_err / f_df");
  if (V == 0 || P == 0) return TFCE_OK;
  tfgb::RmTable tb{};
  for (int r = 0; r < n_rows; ++r) {
    TFGB_CHECK_ARG(row_off[r] >= 0 && row_pstride[r] >= 0, "negative ESS offset");
    tb.row_off[r] = row_off[r];
    tb.row_pstride[r] = row_pstride[r];
  }
  for (int i = 0; i < n_eb; ++i) {
    TFGB_CHECK_ARG(eb_rows && eb_rows[i] >= 0 && eb_rows[i] < n_rows, "between-subject error row out of range");
    tb.eb_rows[i] = eb_rows[i];
  }
  for (int i = 0; i < n_ew; ++i) {
    TFGB_CHECK_ARG(ew_rows && ew_rows[i] >= 0 && ew_rows[i] < n_rows, "within-subject error row out of range");
    tb.ew_rows[i] = ew_rows[i];
  }
  for (int f = 0; f < n_f; ++f) {
    TFGB_CHECK_ARG(f_num[f] >= 0 && f_num[f] < n_rows, "F numerator row out of range");
    TFGB_CHECK_ARG(f_err[f] == 0 || f_err[f] == 1, "F error term must be 0 or 1");
    tb.f_num[f] = f_num[f];
    tb.f_err[f] = f_err[f];
    tb.f_df[f] = f_df[f];
  }
  tb.n_eb = n_eb;
  tb.n_ew = n_ew;
  tb.n_f = n_f;
  tb.df_b = df_b;
  tb.df_w = df_w;
  const int smem = N * tfgb::kRmTile * static_cast<int>(sizeof(float));
  TFGB_CUDA(cudaFuncSetAttribute(tfgb::rm_anova_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  const dim3 grid(static_cast<unsigned>((V + tfgb::kRmTile - 1) / tfgb::kRmTile),
                  static_cast<unsigned>((P + tfgb::kRmPermsPerBlock - 1) / tfgb::kRmPermsPerBlock));
  tfgb::rm_anova_kernel<<<grid, tfgb::kRmThreads, smem, static_cast<cudaStream_t>(stream)>>>(
      Y, ldy, N, V, rows, P, goff, n_groups, ess, tb, out, ldo, ss_out, err);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

}  // extern "C"
