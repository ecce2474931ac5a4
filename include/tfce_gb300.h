/*
 * tfce_gb300.h -- C-ABI of the GB300 permutation-inference path.
 *
 * Plain pointers and sizes only.  "Host" arguments are ordinary host memory;
 * "device" arguments are CUDA device pointers on the current device; `stream`
 * is a cudaStream_t passed as void* (NULL = legacy default stream).  Every
 * entry point returns a tfce_status; tfce_last_error() gives the message of the
 * last failure on the calling thread.
 *
 * Reference interfaces replaced (paths inside trislett/TFCE_mediation):
 *   CreateAdjSet.__init__  tfce_mediation/tfce.pyx:30-42   -> tfce_adjset_create
 *   CreateAdjSet.run       tfce_mediation/tfce.pyx:44-45   -> tfce_adjset_run
 *     (the sweep itself:   tfce_mediation/lib/fast_tfce.hpp:11-95)
 *   write_perm_maxTFCE_vertex / _voxel  tfce_mediation/pyfunc.py:107-126,
 *   write_vertStat_img / write_voxelStat_img  tfce_mediation/pyfunc.py:80-103,
 *   tm_func.calculate_tfce / low_ram_calculate_tfce  tfce_mediation/tm_func.py:54-185
 *                                                     -> tfce_sweep_batch
 *   tval_int + se_of_slope  tfce_mediation/cynumstats.pyx:47-64,
 *   calc_beta_se            tfce_mediation/cynumstats.pyx:66-74  -> glm_tstat (FP32, permutations),
 *                                                                   glm_stat_f64 (observed, helpers)
 *   calc_sobelz / calc_indirect  tfce_mediation/pyfunc.py:130-162,2678-2709
 *                                                     -> sobel_combine
 *   calculate_fweP_vertex.find_nearest  tfce_mediation/tmanalysis/calculate_fweP_vertex.py:37-69,
 *   calculate_fweP_voxel.find_nearest   tfce_mediation/tmanalysis/calculate_fweP_voxel.py:23-49,
 *   tm_func.find_nearest                tfce_mediation/tm_func.py:566-573
 *                                                     -> fwer_sort, fwer_lookup
 *   glm_typeI / glm_cosinor  tfce_mediation/pyfunc.py:2282-2560  -> glm_stat_tc (modes 1-3)
 *   reg_rm_ancova_one_bs_factor / _two_bs_factor  tfce_mediation/pyfunc.py:1712-2280
 *                                                     -> glm_stat_tc (mode 4), rm_anova_combine
 *   calc_gd_fwhm  tfce_mediation/cynumstats.pyx:76-107  -> gd_fwhm_weights, gd_fwhm_smooth
 *   adjacency.compute / compute_distance_parallel  tfce_mediation/adjacency.pyx:44-106
 *                                                     -> geodesic_mesh_*, geodesic_distance_lists
 */
#ifndef TFCE_GB300_H_
#define TFCE_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  TFCE_OK = 0,
  TFCE_EINVAL = 1,    /* bad argument (null pointer, size, adjacency index)  */
  TFCE_EDEVICE = 2,   /* CUDA runtime error                                    */
  TFCE_ETIMEOUT = 3,  /* a bounded device loop hit its iteration limit         */
  TFCE_ENOMEM = 4,    /* device allocation failed                              */
  TFCE_ERANGE = 5     /* more thresholds than the sweep supports (maxT ~ 0)    */
} tfce_status;

/* Library version (major*10000 + minor*100 + patch). */
int tfce_version(void);
/* Message of the last failure on this thread ("" if none). */
const char* tfce_last_error(void);

/* ---------------------------------------------------------------------------
 * Adjacency sets.  A handle owns a device CSR over V vertices, optionally cut
 * into segments (hemispheres, surfaces of a multisurface study).  Entry b in
 * the list of a means "a is adjacent to b" exactly as the reference's
 * adjacencyList[a] (tfce_mediation/tfce.pyx:30-42).  Entries that point
 * outside [0, V) are rejected; self entries are dropped (the reference never
 * unions a vertex with itself); entries whose reverse is missing are marked so
 * the sweep applies the reference's insertion-order rule to them.
 * ------------------------------------------------------------------------- */
typedef struct tfce_adjset tfce_adjset;

/* Host CSR (offsets[V+1], indices[offsets[V]]).  Segments: seg_offsets
 * [n_seg+1] with seg_offsets[0] = 0, seg_offsets[n_seg] = V, or NULL for one
 * segment; adjacency must not cross segments.  H, E: per-segment TFCE
 * parameters (arrays of n_seg), as CreateAdjSet(H, E, adjacency) stores them. */
int tfce_adjset_create(const int64_t* offsets, const int32_t* indices, int32_t n_vertices,
                       const int64_t* seg_offsets, int32_t n_seg, const float* H,
                       const float* E, tfce_adjset** out);
void tfce_adjset_destroy(tfce_adjset* h);
/* Replace the per-segment H/E (host arrays of n_seg). */
int tfce_adjset_set_params(tfce_adjset* h, const float* H, const float* E);
/* 1 if every entry has its reverse (the usual triangle-mesh / 26-neighbour
 * case), 0 otherwise. */
int tfce_adjset_is_symmetric(const tfce_adjset* h);
/* CTA shape of the per-component sweeps (tfce_sweep_batch with
 * accumulation 1 or 2): 3 resident CTAs of 512 threads per SM (40 registers,
 * the most sweeps in flight; the default) or 2 (64 registers, no spills).
 * The autotuner picks it per study together with the batch size. */
int tfce_adjset_set_sweep_shape(tfce_adjset* h, int32_t ctas_per_sm);
/* Threshold groups of tfce_sweep_batch: group [n_seg] (host; ids in
 * [0, n_seg)), or NULL to give every segment its own table again.  Segments
 * of one group share one threshold table per (map, sign), built from the
 * largest maximum among them -- the sweep of tm_func.calculate_tfce
 * (tfce_mediation/tm_func.py:68-78) over one merged adjacency of several
 * surfaces (merge_adjacency_array, tm_func.py:521-540), whose dT is the
 * merged image's max / 100, while each surface is still scaled by its own
 * max / 100 (tm_func.py:84-91).  calc_mixed_tfce (tm_func.py:327-378) is one
 * group per TFCE setting.  A grouped launch adds one segment-maximum pass
 * over the maps. */
int tfce_adjset_set_threshold_groups(tfce_adjset* h, const int32_t* group);

/* How tfce_sweep_batch accumulates (the other entry points always use 0):
 *   0  the reference's arithmetic: every active vertex adds its float
 *      increment to a float accumulator at every threshold
 *      (fast_tfce.hpp:72-84), so results are bit-identical to the reference
 *      up to its libm's powf rounding (the default);
 *   1  per-component: each live component adds its increment once per
 *      threshold in double, and a vertex's value is resolved at the end along
 *      the chain of components it joined; the value is the float rounding of
 *      the exact sum of the same float increments, i.e. it differs from the
 *      reference by the reference's own float summation error (~1e-7 rel).
 *      Work per threshold is O(live components) instead of O(active vertices).
 *      A launch that asks only for maxima (out_maps NULL) without vertex
 *      weights (vdensity NULL) keeps, per component, the largest sum of any
 *      component merged into it instead of the potentials, and takes the
 *      map's maximum over the last live components: no per-vertex pass;
 *   2  as 1, but maxima-only launches keep the potentials and resolve every
 *      vertex as well (the same values; for comparisons). */
int tfce_adjset_set_accumulation(tfce_adjset* h, int32_t mode);

/* CreateAdjSet.run(image, enhn) on host float32 arrays of length V (one
 * segment: the whole handle).  Accumulates the sweep into enhn, as
 * fast_tfce.hpp:82 does.  Synchronous. */
int tfce_adjset_run(tfce_adjset* h, const float* image, float* enhn, int32_t n_vertices);

/* Debug sweep of one host map through the device kernel, recording per
 * threshold the component label (root vertex id, -1 inactive) and extent of
 * every vertex: labels/extents are host arrays of max_steps*V; *n_steps gets
 * the number of thresholds.  One segment handles only.  Synchronous. */
int tfce_adjset_run_labels(tfce_adjset* h, const float* image, float* enhn, int32_t n_vertices,
                           int32_t* labels, int32_t* extents, int32_t max_steps,
                           int32_t* n_steps);

/* Batched sweep (device pointers, stream-ordered).
 *   stats     [n_maps][map_stride] floats, the statistic of every map laid out
 *             over the handle's V vertices (segment s = [seg_off[s], seg_off[s+1]));
 *   signs     1 = (+), 2 = (+,-) : every map is swept as +stat and, with 2, as -stat;
 *   vdensity  [V] per-vertex weight or NULL (weight 1);
 *   floor_zero nonzero: each segment's maximum is taken as at least 0, as when
 *             a masked statistic is scattered into a zero-filled surface;
 *   out_max   [n_maps][signs][n_seg]: max over the segment of
 *             TFCE * (segment max / 100) * vdensity (pyfunc.py:116-118);
 *   out_maps  [n_maps][signs][V] or NULL; out_mode 1 writes the scaled map,
 *             out_mode 2 adds the raw sweep into out_maps (enhn semantics).
 * Uses a device workspace that the handle grows on demand. */
int tfce_sweep_batch(tfce_adjset* h, const float* stats, int64_t map_stride, int32_t n_maps,
                     int32_t signs, const float* vdensity, int32_t floor_zero, float* out_max,
                     float* out_maps, int32_t out_mode, void* stream);
/* Synchronises `stream`, then returns (and clears) the device error word that
 * the batched sweeps queued on this handle since the last call have set:
 * TFCE_EINVAL (entry outside its segment), TFCE_ETIMEOUT (iteration limit),
 * TFCE_ERANGE (threshold table overflow). */
int tfce_sweep_status(tfce_adjset* h, void* stream);
/* Sweep items the batched sweep runs at once on the handle's device: its
 * persistent grid (resident CTAs per SM x SMs; TFCE_SWEEP_MAX_CTAS caps it).
 * A launch of n items runs in ceil(n / slots) waves. */
int tfce_sweep_resident_slots(tfce_adjset* h, int32_t* slots);

/* Allocation-free form of tfce_sweep_batch.  No counterpart in the reference.
 *
 * For callers that cannot allocate device memory while they sweep: a host
 * whose device memory is reserved up front by another allocator, a real-time
 * loop that must keep a fixed footprint, or a program that cannot take the
 * device-wide synchronisation that cudaFree implies.  Nothing is allocated:
 * no handle, no cudaMalloc/cudaFree.  The scratch is a 64 MiB static device
 * array inside this library, which every process that loads the library holds
 * on each GPU it uses until exit.
 *
 *   offsets [n_vertices+1] (int64), indices [n_entries] (int32): the caller's
 *     adjacency, already on the device, in the same CSR form tfce_adjset_create
 *     takes (it need not be symmetric; self entries are allowed);
 *   seg_offsets [n_seg+1] (device int64), H/E [n_seg] (device float);
 *   max_segment_vertices: an upper bound on the vertex count of every segment;
 *     at most 2,796,160 (what one workspace slot of the 64 MiB holds) --
 *     larger values return TFCE_ERANGE before any device work; a segment
 *     found larger on the device returns TFCE_EINVAL;
 *   stats, map_stride, n_maps, signs, vdensity, floor_zero, out_max: as
 *     tfce_sweep_batch (device pointers; only the maxima are written).
 * Every call looks up the array's device address in the current context
 * (cudaGetSymbolAddress) with the caller's device current.  The call is
 * synchronous: it returns when the sweeps have finished (it copies the error
 * word back and synchronises `stream`) with the device status, so it cannot
 * be called while `stream` is being captured into a CUDA graph.  All calls
 * share the one array, which keeps the last call's contents (the queue and
 * error words are cleared on entry): calls that overlap on the GPU -- from
 * two threads, or on two streams -- race.  A negative list entry, an entry
 * outside its segment or a segment longer than max_segment_vertices makes
 * the call return TFCE_EINVAL; the item it belongs to then reports 0 (a
 * segment too long) or is swept without that entry. */
int tfce_sweep_batch_noalloc(const int64_t* offsets, const int32_t* indices, int32_t n_vertices,
                             int64_t n_entries, const int64_t* seg_offsets, int32_t n_seg,
                             int32_t max_segment_vertices, const float* H, const float* E,
                             const float* stats, int64_t map_stride, int32_t n_maps,
                             int32_t signs, const float* vdensity, int32_t floor_zero,
                             float* out_max, void* stream);

/* ---------------------------------------------------------------------------
 * Mass-univariate OLS t for G designs against one data matrix (device).
 *   Y       [n][ldy] float32, subjects x vertices (merge_y layout), V columns used;
 *   pinv    [G][kmax][n]  rows of inv(X'X)X' (rows >= k_g zero), float32;
 *   X       [G][n][kmax]  the (permuted) design, columns >= k_g zero;
 *   invdiag [G][kmax]     diag(inv(X'X));
 *   dof     [G]           n - k_g;
 *   coef    [n_coef]      coefficient indices written for every design;
 *   t_out   [G][n_coef][ldt].
 * beta = pinv.y, RSS from the residuals y - X.beta (never from Y'Y),
 * se = sqrt(RSS/dof * invdiag), t = beta / se  (cynumstats.pyx:28-29,47-64). */
int glm_tstat(const float* Y, int64_t ldy, int32_t n, int64_t V, const float* pinv,
              const float* X, const float* invdiag, const float* dof, int32_t G, int32_t kmax,
              const int32_t* coef, int32_t n_coef, float* t_out, int64_t ldt, void* stream);

/* The same fit with another output (`what`), for the one-off helpers of
 * tfce_mediation/cynumstats.pyx:
 *   0 t [G][n_coef][ldo]          (tval_int, :59-64)
 *   1 beta [G][n_coef][ldo]       (cy_lin_lstsqr_mat, :28-29; calc_beta_se, :66-74)
 *   2 se [G][n_coef][ldo]         (se_of_slope, :47-52)
 *   3 residuals [G][n][ldo]       (resid_covars, :54-57)
 *   4 F [G][ldo], k_g = n - dof_g, TSS about each column's mean
 *                                 (glm_fstat gives the reference's centring)
 *   5 RSS [G][ldo]                (cy_lin_lstsqr_mat_residual, :109-112)
 * coef/invdiag may be NULL where the output does not use them. */
int glm_stat(const float* Y, int64_t ldy, int32_t n, int64_t V, const float* pinv,
             const float* X, const float* invdiag, const float* dof, int32_t G, int32_t kmax,
             const int32_t* coef, int32_t n_coef, int32_t what, float* out, int64_t ldo,
             void* stream);

/* The same fit in FP64 with the reference's precision (the observed
 * statistic and the one-off helpers): betas and sigma^2 in double from the
 * float32 data, the SE rounded to float32 as se_of_slope stores it
 * (tfce_mediation/cynumstats.pyx:47-52), t = double beta / that SE
 * (tval_int, :59-64).  pinv [G][kmax][n], X [G][n][kmax], invdiag [G][kmax],
 * dof [G] are double; what 0 = t, 1 = beta, 2 = SE; out [G][n_coef][ldo]
 * double.  G <= 65535; 2 * kmax * n doubles must fit in 200 KB of shared
 * memory (n <= 1600 at kmax = 8). */
int glm_stat_f64(const float* Y, int64_t ldy, int32_t n, int64_t V, const double* pinv, const double* X,
                 const double* invdiag, const double* dof, int32_t G, int32_t kmax, const int32_t* coef,
                 int32_t n_coef, int32_t what, double* out, int64_t ldo, void* stream);

/* Model F as calcF computes it (tfce_mediation/cynumstats.pyx:31-36):
 * ((TSS - RSS)/(k_g-1)) / (RSS/dof_g) with TSS taken around *centre (a device
 * float; the reference centres on np.mean(y), the grand mean of the whole
 * matrix), or around each column's mean when centre is NULL.  f_out [G][ldf]. */
int glm_fstat(const float* Y, int64_t ldy, int32_t n, int64_t V, const float* pinv,
              const float* X, const float* dof, int32_t G, int32_t kmax, const float* centre,
              float* f_out, int64_t ldf, void* stream);

/* Tensor-core (tcgen05) form of glm_tstat (same t as cynumstats.pyx:28-64),
 * split BF16: every GEMM operand is hi = bf16(x), lo = bf16(x - hi);
 * beta = Y_hi.P_hi + Y_hi.P_lo + Y_lo.P_hi with FP32 accumulation in tensor
 * memory (three tcgen05.mma per 16-deep step; M = 128 vertices, N = 8 rows
 * per design), then the residuals y - X.beta (FP32 data), RSS, SE and t on
 * the CUDA cores.
 *   glm_tc_design_block(kmax): designs per tile DB (32 for kmax <= 5, else
 *     16); -1 for kmax outside [1, 8];
 *   glm_tile_bytes(rows, row_block, n_pad): bytes of a pre-tiled operand;
 *   glm_col_mean: mean[v] = FP64 mean over the n rows of Y [n][ldy] (the
 *     per-vertex centre of the data);
 *   glm_tile_split: dst = the split-BF16 tiles of src [rows][cols] (row
 *     stride ld_src; transpose = 1: src stored [cols][rows], the data n x V)
 *     minus row_shift[row] when row_shift is not NULL, in row blocks of
 *     row_block (128 for the data, DB*8 for the stacked pseudoinverse rows
 *     [G_pad*8][n_pad], rows >= k_g of a design zero) and 16-deep K steps,
 *     n_pad a multiple of 16 >= cols, zero fill; shifted (optional) receives
 *     src minus row_shift as FP32 in src's layout (the centred data);
 *   glm_tstat_tc: y_tiles (row block 128, centred on y_shift when that is not
 *     NULL) and p_tiles (row block DB*8) from glm_tile_split; u_rows
 *     [G_pad][kmax] = pinv(X_d).1 (needed with y_shift: beta = beta_c +
 *     y_shift[v] u_d); Y the FP32 data [n][ldy]; x_rows
 *     [ceil(G/DB)][n_sc][kmax][DB] float, the NEGATED design rows (design d of
 *     block b, row i at [b][i][j][d], zero padded; n_sc a multiple of 32 >= n);
 *     invdiag / dof / coef / t_out as glm_tstat; err: a device int32 that
 *     receives TFCE_ETIMEOUT's device code if a copy or MMA completion wait
 *     runs out (all are bounded).  Tiles and x_rows 16-byte aligned. */
int glm_tc_design_block(int32_t kmax);
int64_t glm_tile_bytes(int64_t rows, int32_t row_block, int32_t n_pad);
int glm_col_mean(const float* Y, int64_t ldy, int32_t n, int64_t V, float* mean, void* stream);
int glm_tile_split(const float* src, int64_t ld_src, int32_t transpose, int64_t rows, int32_t cols,
                   const float* row_shift, int32_t row_block, int32_t n_pad, void* dst, float* shifted,
                   void* stream);
int glm_tstat_tc(const void* y_tiles, const float* y_shift, const float* Y, int64_t ldy, int32_t n,
                 int32_t n_pad, int64_t V, const void* p_tiles, const float* u_rows, const float* x_rows,
                 int32_t n_sc, const float* invdiag, const float* dof, int32_t G, int32_t kmax,
                 const int32_t* coef, int32_t n_coef, float* t_out, int64_t ldt, int32_t* err, void* stream);
/* glm_stat_tc: glm_tstat_tc with a choice of epilogue output (t_out rows [G][n_coef][ldt]):
 *   mode 0: t of the coefficients coef[0..n_coef) (= glm_tstat_tc);
 *   mode 1: RSS from the residuals, one row per design (n_coef, coef ignored);
 *   mode 2: partial F of n_coef column groups, coef = (start, width) pairs over
 *     the design's columns: F = (RSS without the group - RSS) / width / (RSS/dof),
 *     the reference's glm_typeI drop-one F (tm/pyfunc.py:2282-2400), with the
 *     extra sum of squares in its exact form b_S' inv(inv(X'X)_SS) b_S; wmat
 *     [G][w_stride] holds, per design, the groups' inv(inv(X'X)_SS) blocks
 *     (row-major, concatenated in group order).  A group outside [0, kmax)
 *     yields NaN.
 *   mode 3: a program of n_coef typed output rows, coef = 4 int32 per row
 *     (kind, column j, width w, offset o into the design's wmat row):
 *       kind 0: t of coefficient j;  kind 1: -t of coefficient j (the
 *         reference sweeps -t as its own map);
 *       kind 2: partial F of the columns [j, j+w), inv(inv(X'X)_SS) at o (w*w);
 *       kind 3 / 4: the cosinor amplitude / acrophase t of the pair (j, j+1)
 *         = (cos, sin) coefficients (glm_cosinor, tm/pyfunc.py:2406-2560),
 *         inv(X'X) entries (jj, j j+1, j+1 j+1) at o: with A^2 = b_j^2 + b_j+1^2
 *         and sigma^2 = RSS/dof, A^2 / (sigma sqrt(I11 b_j^2 -/+ 2 I12 |b_j b_j+1|
 *         + I22 b_j+1^2)) for the amplitude (-) and with b_j, b_j+1 swapped
 *         (+) for the acrophase -- the reference's error propagation through
 *         |sin|, |cos| of arctan(|b_j+1 / b_j|).
 *       kind 5: the extra sum of squares of dropping the columns [j, j+w),
 *         b_S' inv(inv(X'X)_SS) b_S with the block at o (w*w) (kind 2 without
 *         its division by w and RSS/dof);
 *     A row whose columns or weights fall outside kmax / w_stride yields NaN.
 *   mode 4: a program of kind-5 rows only, without the residual pass: x_rows,
 *     invdiag, dof and Y_centred may be NULL (the "designs" may then be any
 *     stacks of up to kmax pseudoinverse rows, e.g. the column blocks of
 *     several designs); rows of other kinds yield NaN.
 *     The model F of glm_cosinor / glm_typeI is kind 2 over every column
 *     after the intercept.
 *   Y_centred (optional): Y minus its per-vertex centre (glm_col_center with
 *     y_shift); only for designs whose first column is all ones and whose
 *     x_rows hold the other columns minus their means: the residuals are then
 *     formed without the intercept term (one FMA fewer per vertex, design and
 *     subject); coefficient 0 is then not available (t of it, or a group
 *     holding it, is returned as 0). */
int glm_col_center(const float* Y, int64_t ldy, int32_t n, int64_t V, const float* centre, float* out,
                   void* stream);
/* glm_stat_tc with the tile's design count chosen: design_block 32 (N = 256
 * MMA columns, kmax <= 5; the default there) or 16 (N = 128; the only choice
 * for kmax > 5), 0 = the default (glm_tc_design_block).  p_tiles and x_rows
 * must be laid out for the same design_block (row blocks of design_block * 8
 * pseudoinverse rows; x_rows [ceil(G / design_block)][n_sc][kmax][design_block]).
 * The autotuner times both for designs with kmax <= 5. */
int glm_stat_tc_block(const void* y_tiles, const float* y_shift, const float* Y, const float* Y_centred,
                      int64_t ldy, int32_t n, int32_t n_pad, int64_t V, const void* p_tiles, const float* u_rows,
                      const float* x_rows, int32_t n_sc, const float* invdiag, const float* dof, int32_t G,
                      int32_t kmax, int32_t design_block, int32_t mode, const int32_t* coef, int32_t n_coef,
                      const float* wmat, int32_t w_stride, float* t_out, int64_t ldt, int32_t* err, void* stream);
/* Permutation index streams of the mmr-lr convention (tm_func.py:147-151):
 * out[(p - start) * n + i] = numpy.random.RandomState(seed + p).permutation(n)[i]
 * for p in [start, stop), bit for bit (MT19937 seeded from one 32-bit
 * integer, Fisher-Yates from the last element with masked-rejection draws).
 * Host work only, split over `threads` threads (0 = the hardware count).
 * TFCE_EINVAL when a seed + p falls outside [0, 2^32 - 1] (RandomState's
 * own range). */
int perm_stream(int64_t n, int64_t seed, int64_t start, int64_t stop, int64_t* out, int32_t threads);

/* Quadratic-form tensor-core GLM: t of coefficients >= 1 of designs whose
 * first column is all ones (the same t as cynumstats.pyx:28-64 / glm_tstat).
 * By Frisch-Waugh, with Xc the other columns minus their means and c =
 * Xc'(y - centre) from one split-BF16 GEMM (M = 128 vertices, N = 256: R = 4
 * rows per design for kmax <= 5, 8 for kmax <= 8):
 *   b = inv(Xc'Xc) c,  RSS = yy - c'b,  t_j = b_j / sqrt(RSS / dof * invdiag_j);
 * no residual pass over the subjects.
 *   glm_qf_design_block(kmax): designs per tile (64 for kmax <= 5, 32 for
 *     kmax <= 8); -1 for kmax outside [2, 8];
 *   glm_col_sumsq: yy[v] = sum_i (Yc[i][v] - mean_v)^2 over the n rows of the
 *     centred data (glm_tile_split's `shifted` output), FP64 accumulation;
 *   glm_tstat_tc_qf: y_tiles as glm_tstat_tc (centred); x_tiles from
 *     glm_tile_split of the centred design columns stacked [G_pad*R][n_pad]
 *     (design d, column j >= 1 at row d*R + j - 1, other rows zero) in row
 *     blocks of 256; ginv [G_pad][R][R] = inv(X'X) without its first row
 *     and column (= inv(Xc'Xc)), zero padded to R x R; invdiag [G][kmax]
 *     and dof [G] as glm_tstat; coef[0..n_coef), n_coef <= 8, in [1, kmax)
 *     (another index yields NaN); err as glm_tstat_tc.  RSS is clamped at 0
 *     (a perfect fit gives +-inf or NaN, as 0/0).  Tiles and ginv 16-byte
 *     aligned. */
int glm_qf_design_block(int32_t kmax);
int glm_col_sumsq(const float* Y_centred, int64_t ldy, int32_t n, int64_t V, float* yy, void* stream);
int glm_tstat_tc_qf(const void* y_tiles, const float* yy, int32_t n, int32_t n_pad, int64_t V,
                    const void* x_tiles, const float* ginv, const float* invdiag, const float* dof, int32_t G,
                    int32_t kmax, const int32_t* coef, int32_t n_coef, float* t_out, int64_t ldt, int32_t* err,
                    void* stream);
int glm_stat_tc(const void* y_tiles, const float* y_shift, const float* Y, const float* Y_centred, int64_t ldy,
                int32_t n,
                int32_t n_pad, int64_t V, const void* p_tiles, const float* u_rows, const float* x_rows,
                int32_t n_sc, const float* invdiag, const float* dof, int32_t G, int32_t kmax, int32_t mode,
                const int32_t* coef, int32_t n_coef, const float* wmat, int32_t w_stride, float* t_out,
                int64_t ldt, int32_t* err, void* stream);

/* Indirect-effect z from path t values (device), z[p][v] for p < P:
 *   ta [P][lda] (or ta_scalar[P] when ta is NULL: medtype Y's linregress path),
 *   tb [P][ldb];  alg 0 = Aroian, 1 = Sobel, 2 = Goodman (pyfunc.py:146-161). */
int sobel_combine(const float* ta, int64_t lda, const float* ta_scalar, const float* tb,
                  int64_t ldb, int32_t P, int64_t V, int32_t alg, float* z, int64_t ldz,
                  void* stream);

/* ---------------------------------------------------------------------------
 * Repeated-measures ANCOVA (reg_rm_ancova_one_bs_factor /
 * reg_rm_ancova_two_bs_factor, tm/pyfunc.py:2067-2280 and 1712-2060, as
 * tm_models_randomise.py:522-684 permutes them).  The effect sums of squares
 * come from glm_stat_tc mode 4 (kind 5 rows: extra sums of squares in Wald
 * form); rm_anova_combine forms, per permutation p and vertex v, the sums of
 * squares between and within subject means of the permuted data and the F maps:
 *   Y       [N][ldy] data (device; centring per vertex is recommended);
 *   rows    [P][N] int32 (device): data rows of permutation p grouped by
 *           subject, group g = rows[p][goff[g] .. goff[g+1]);
 *   goff    [n_groups+1] int32 (device);
 *   ess     device base of the sums-of-squares rows: row r of permutation p
 *           at ess[row_off[r] + p * row_pstride[r] + v] (row_off, row_pstride:
 *           host arrays of n_rows <= 16);
 *   error terms: between = SS_between - sum of rows eb_rows[0..n_eb),
 *                within  = SS_within  - sum of rows ew_rows[0..n_ew)  (host arrays);
 *   F map f (n_f <= 8; host arrays): (ess row f_num[f] / f_df[f]) /
 *           (error f_err[f] (0 between, 1 within) / df_b or df_w);
 *   out     [P][n_f][ldo]; ss_out (optional) [P][2][ldo]: SS_between, SS_within.
 * N <= rm_anova_max_rows() (the kernel stages all N rows of a 32-vertex tile).
 * A row index or group bound out of range sets *err (device) to 1 and is clamped. */
int rm_anova_max_rows(void);
int rm_anova_combine(const float* Y, int64_t ldy, int32_t N, int64_t V, const int32_t* rows, int32_t P,
                     const int32_t* goff, int32_t n_groups, const float* ess, const int64_t* row_off,
                     const int64_t* row_pstride, int32_t n_rows, const int32_t* eb_rows, int32_t n_eb,
                     const int32_t* ew_rows, int32_t n_ew, float df_b, float df_w, const int32_t* f_num,
                     const int32_t* f_err, const float* f_df, int32_t n_f, float* out, int64_t ldo, float* ss_out,
                     int32_t* err, void* stream);

/* ---------------------------------------------------------------------------
 * Geodesic FWHM smoothing (calc_gd_fwhm, tm/cynumstats.pyx:76-107, as
 * tools/tm_gd_fwhm_smoothing.py:96 calls it per subject image).
 * gd_fwhm_weights: w[x] = pdf_compute(dist[x], 0, scale) for x < M and the
 *   self weight pdf_compute(0, 0, scale) at w[M] (device arrays; w has M+1).
 * gd_fwhm_smooth: B images data [B][ld] over V vertices -> out [B][ldo]:
 *   out[v] = (sum_k w[pidx[k]] * data[src[k]] + w[M] * data[v]) /
 *            (sum_k w[pidx[k]] + w[M]) over k in [off[v], off[v+1]),
 *   float32 with one rounding per product and per sum, in k order.  The gather
 *   list (device: off [V+1] int64, src / pidx [off[V]] int32) holds, for every
 *   pair x = (i, j) of the reference's list, the entry (i, x) under vertex j
 *   and (j, x) under vertex i, each vertex's entries in pair order (the order
 *   of the reference's scatter).  An entry outside [0, V) / [0, M) sets *err
 *   (device) to 1 and is skipped. */
int gd_fwhm_weights(const float* dist, int64_t M, float scale, float* w, void* stream);
int gd_fwhm_smooth(const int64_t* off, const int32_t* src, const int32_t* pidx, const float* w, int64_t M,
                   const float* data, int64_t ld, int32_t B, int32_t V, float* out, int64_t ldo, int32_t* err,
                   void* stream);

/* ---------------------------------------------------------------------------
 * Exact geodesic distance lists (adjacency.compute / compute_distance_parallel,
 * tfce_mediation/adjacency.pyx:44-106, over the exact geodesic library in
 * tfce_mediation/lib/geodesic).  For every source vertex i of a triangle mesh,
 * the vertices j whose exact geodesic distance along the surface is below a
 * threshold.  Propagation runs from each source up to threshold + 1e-10, as
 * the reference propagates (adjacency.pyx:54, :94).
 *   geodesic_mesh_create: host pts [n_vertices][3] float32 and faces
 *     [n_faces][3] int32; rejects (TFCE_EINVAL) out-of-range or repeated face
 *     vertices, zero-length edges, zero-area faces and edges shared by more
 *     than two faces.  Vertices whose total angle exceeds 2 pi - 1e-5, and
 *     boundary vertices, are the pseudo-sources geodesics may bend around
 *     (the reference's rule, lib/geodesic/geodesic_mesh.h:335-344);
 *     geodesic_mesh_saddles returns their count.
 *   geodesic_distance_lists: sources [src_lo, src_hi); keeps (i, j, distance)
 *     for every j != i with distance < threshold (only j > i when
 *     only_greater, the pairs compute_distance_parallel returns), sorted by i
 *     then j; *n_out gets their number.  Synchronous.  TFCE_ERANGE when a
 *     source's propagation outgrows 16384 queued windows or reached vertices.
 *   geodesic_take_lists: copies the kept lists into host arrays of at least
 *     *n_out entries and releases them. */
typedef struct geodesic_mesh geodesic_mesh;
int geodesic_mesh_create(const float* pts, int32_t n_vertices, const int32_t* faces, int32_t n_faces,
                         geodesic_mesh** out);
void geodesic_mesh_destroy(geodesic_mesh* m);
int geodesic_mesh_saddles(geodesic_mesh* m, int32_t* n_saddle);
int geodesic_distance_lists(geodesic_mesh* m, double threshold, int32_t only_greater, int32_t src_lo,
                            int32_t src_hi, int64_t* n_out);
int geodesic_take_lists(geodesic_mesh* m, int32_t* out_i, int32_t* out_j, double* out_d, int64_t cap);

/* ---------------------------------------------------------------------------
 * FWER.  fwer_sort sorts n doubles ascending in place (device).  fwer_lookup
 * maps every value of an image through the sorted null of length N (the
 * reference reads its null back from CSV text as float64):
 *   mode 0 (calculate_fweP_*): 1-p = max(idx-1,0)/N with idx = #{null < x},
 *           written only where x > 0 (0 elsewhere);
 *   mode 1 (tm_func.find_nearest): p_array of the nearer neighbour rank,
 *           for every value.
 * image and out are double [V] (device). */
int fwer_sort(double* values, int64_t n, void* stream);
int fwer_lookup(const double* sorted_null, int64_t N, const double* image, int64_t V,
                int32_t mode, double* out, void* stream);

/* ---------------------------------------------------------------------------
 * Learned null-tail surrogate: kernels of a small MLP (no counterpart in the
 * reference, whose only tail model is the gamma / Johnson-SB fit of
 * bin/tm_maths:522-553).  Row-major matrices, device pointers.
 *   mlp_gemm:      C[M][N] = op(A)[M][K] . op(B)[K][N] (+ bias[N]) (+ C when
 *                  accumulate); act 1 applies GELU (erf form) and stores the
 *                  pre-activation in preact (nullable);
 *   mlp_gemm_bf16: forward GEMM with bfloat16 A and B, FP32 accumulation;
 *   mlp_to_bf16:   float -> bfloat16 (round to nearest even);
 *   mlp_gelu_backward: dz = dy * GELU'(z);
 *   mlp_bias_grad: db[c] = sum_r dz[r][c];
 *   mlp_mse_loss:  loss = mean(w_c (y - t)^2), dy = 2 w_c (y - t) / n;
 *   mlp_adam_step: Adam with bias correction and decoupled weight decay. */
int mlp_gemm(int32_t transA, int32_t transB, int32_t M, int32_t N, int32_t K, const float* A,
             int32_t lda, const float* B, int32_t ldb, float* C, int32_t ldc, const float* bias,
             int32_t act, float* preact, int32_t accumulate, void* stream);
int mlp_gemm_bf16(int32_t transA, int32_t transB, int32_t M, int32_t N, int32_t K, const void* A,
                  int32_t lda, const void* B, int32_t ldb, float* C, int32_t ldc, const float* bias,
                  int32_t act, void* stream);
int mlp_to_bf16(const float* x, void* y, int64_t n, void* stream);
int mlp_gelu_backward(const float* dy, const float* z, float* dz, int64_t n, void* stream);
int mlp_bias_grad(const float* dz, int32_t rows, int32_t cols, float* db, void* stream);
int mlp_mse_loss(const float* y, const float* t, const float* col_weight, int64_t n, int32_t cols,
                 float* dy, float* loss, void* stream);
int mlp_adam_step(float* param, const float* grad, float* m, float* v, int64_t n, float lr,
                  float beta1, float beta2, float eps, int32_t step, float weight_decay,
                  void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TFCE_GB300_H_ */
