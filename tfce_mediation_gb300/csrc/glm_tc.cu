// Tensor-core (tcgen05) form of the permuted-design GLM.
//
// One launch computes t maps for G designs over V vertices:
//   beta_d = pinv(X_d) y            (cynumstats.pyx:28-29, np.dot(pinv, y))
//   r      = y - X_d beta_d         (cynumstats.pyx:47-64: the residuals)
//   t      = beta_j / sqrt(r'r / dof * inv(X'X)_jj)
// The betas of all designs are one GEMM, D[v][d*8+j] = sum_i Y[v][i] P[d*8+j][i],
// with M = 128 vertices (tensor-memory lanes), N = 8 pseudoinverse rows per
// design (up to 32 designs: N = 256), K = subjects.  The epilogue forms the
// residuals from y and X_d on the CUDA cores (RSS from the residuals, never
// from Y'Y) and writes t.
//
// Precision: split BF16.  Both operands are stored as hi = bf16(x) and
// lo = bf16(x - hi); each 16-deep K step issues hi.hi + hi.lo + lo.hi
// (tcgen05.mma kind::f16, FP32 accumulation in tensor memory).  The dropped
// lo.lo term and the split's rounding are ~2^-17 relative per product.  The
// residual pass reads the FP32 data.  The data is centred per vertex (FP64
// mean) before the split, so the split error scales with the data's spread,
// not its mean; the epilogue restores beta = beta_c + mean_v * pinv(X_d).1,
// which is exact for any design.
//
// Operands are pre-tiled in HBM (glm_tile_split) so that one K step of a
// tile is a contiguous chunk: one cp.async.bulk per operand per pipeline
// stage, completing on an mbarrier.  In shared memory each chunk is the
// K-major no-swizzle layout of 8-row x 16-byte core matrices:
//   [hi|lo][k-block 0..1][row][8 elements]
// so a descriptor has LBO (next 8 K elements) = rows*16 bytes and SBO (next
// 8 rows) = 128 bytes.
//
// Per CTA (256 threads, 2 CTAs per SM so one CTA's MMAs overlap the other's
// epilogue): thread 0 runs the 4-stage copy/MMA pipeline.  The accumulator is
// then drained (warp w reads TMEM lanes 32*(w%4).., design half w/4) into
// shared memory and re-read transposed: lane = design, each thread a run of
// DB/2 vertices with their betas in registers.  Subjects stream through
// shared memory in chunks of 32 (cp.async, double buffered): the design rows
// are a conflict-free per-lane load, y a broadcast; residual and RSS use
// packed FP32x2 FMAs over vertex pairs.
//
// Every wait is bounded (globaltimer, 2 s): on expiry the kernel records
// kDevLoopLimit in *err, waits (bounded) for its own copies in flight,
// frees its tensor memory and returns.
#include <cuda_bf16.h>

#include <algorithm>

#include "common.cuh"

namespace tfgb {

constexpr int kTcThreads = 256;
constexpr int kTcM = 128;           // vertices per tile (MMA M, TMEM lanes)
constexpr int kTcRowsPerDesign = 8; // pseudoinverse rows per design (kmax <= 8)
constexpr int kTcK = 16;            // subjects per MMA K step / pipeline stage
constexpr int kTcStages = 4;
constexpr int kTcSubjChunk = 32;    // subjects per epilogue X chunk
constexpr uint64_t kTcWaitNs = 2000000000ull;
// output kinds of the programmed epilogue (mode 3)
constexpr int kTcOutT = 0, kTcOutNegT = 1, kTcOutF = 2, kTcOutAmp = 3, kTcOutAcro = 4, kTcOutEss = 5;

// designs per thread in the beta drain: 16 (32-design tiles, N = 256) or 8
// (16-design tiles, N = 128); kmax > 5 always uses 8
__host__ __device__ constexpr int tc_dpt(int kmax) { return kmax <= 5 ? 16 : 8; }
__host__ __device__ constexpr int tc_db(int dpt) { return 2 * dpt; }     // designs per tile
__host__ __device__ constexpr int tc_n(int dpt) { return tc_db(dpt) * kTcRowsPerDesign; }
__host__ __device__ constexpr int tc_y_stage() { return kTcM * kTcK * 2 * 2; }          // 8 KB
__host__ __device__ constexpr int tc_p_stage(int dpt) { return tc_n(dpt) * kTcK * 2 * 2; }
__host__ __device__ constexpr int tc_stage(int dpt) { return tc_y_stage() + tc_p_stage(dpt); }
__host__ __device__ constexpr int tc_xchunk(int kmax, int dpt) { return kTcSubjChunk * kmax * tc_db(dpt) * 4; }
__host__ __device__ constexpr int tc_ychunk() { return kTcSubjChunk * kTcM * 4; }
constexpr int kTcBld = kTcM + 1;  // row stride (floats) of the drained betas
__host__ __device__ constexpr int tc_beta_bytes(int kmax, int dpt) { return tc_db(dpt) * kmax * kTcBld * 4; }
__host__ __device__ constexpr int tc_cmax(int a, int b) { return a > b ? a : b; }
// partial-F epilogue: every thread's betas and RSS (DB/2 vertices x (kmax+1) floats)
__host__ __device__ constexpr int tc_fslice_bytes(int kmax, int dpt) { return 256 * (tc_db(dpt) / 2) * (kmax + 1) * 4; }
// the stage ring, the drained betas, the subject chunks and the partial-F
// slices share one area
__host__ __device__ constexpr int tc_area(int kmax, int dpt) {
  return (tc_cmax(tc_cmax(tc_cmax(kTcStages * tc_stage(dpt), tc_beta_bytes(kmax, dpt)),
                          2 * (tc_xchunk(kmax, dpt) + tc_ychunk())),
                  tc_fslice_bytes(kmax, dpt)) + 127) / 128 * 128;
}
__host__ __device__ constexpr int tc_smem(int kmax, int dpt) { return tc_area(kmax, dpt) + 128; }
static_assert(tc_smem(5, 16) <= 113 * 1024 && tc_smem(8, 8) <= 113 * 1024 && tc_smem(4, 16) <= 113 * 1024 &&
                  tc_smem(5, 8) <= 113 * 1024,
              "two CTAs per SM");


// --- PTX wrappers -----------------------------------------------------------
__device__ inline uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ inline uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// tcgen05 shared-memory matrix descriptor, K-major, no swizzle:
// start >> 4 [0,14), leading (K) byte offset >> 4 [16,30), stride (M/N) byte
// offset >> 4 [32,46), version 1 [46,48), swizzle 0 [61,64).
__device__ inline uint64_t make_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (static_cast<uint64_t>((addr >> 4) & 0x3FFF)) |
         (static_cast<uint64_t>((lbo >> 4) & 0x3FFF) << 16) |
         (static_cast<uint64_t>((sbo >> 4) & 0x3FFF) << 32) | (1ULL << 46);
}

// kind::f16 instruction descriptor: D F32 [4,6)=1, A BF16 [7,10)=1,
// B BF16 [10,13)=1, both K-major, N>>3 at [17,23), M>>4 at [24,29).
__host__ __device__ constexpr uint32_t make_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
         (static_cast<uint32_t>(M >> 4) << 24);
}

__device__ inline void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ inline void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

__device__ inline void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

__device__ inline bool mbar_try_wait(uint32_t mbar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(phase)
      : "memory");
  return ok != 0;
}

// Bounded wait on an mbarrier phase; false when the time limit ran out.
__device__ inline bool mbar_wait(uint32_t mbar, uint32_t phase) {
  if (mbar_try_wait(mbar, phase)) return true;
  const uint64_t t0 = global_ns();
  while (!mbar_try_wait(mbar, phase)) {
    if (global_ns() - t0 > kTcWaitNs) return false;
  }
  return true;
}

__device__ inline void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

__device__ inline void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(mbar)
      : "memory");
}

__device__ inline void cp_async16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ inline void cp_async4(uint32_t dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ inline void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ inline void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ inline void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ inline void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ inline void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ inline void tmem_ld8(uint32_t taddr, float* out) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) out[i] = __uint_as_float(r[i]);
}

__device__ inline void tmem_ld16(uint32_t taddr, float* out) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) out[i] = __uint_as_float(r[i]);
}

// --- operand pre-tiling -------------------------------------------------------
// dst = the split-BF16 tiles of a [rows][cols] FP32 matrix (row stride ld_src;
// transpose: the source is stored [cols][rows], e.g. the data n x V):
//   byte offset of (row R, col c) = ((R/RB * KS + c/16) * 2 + part) * RB*32
//                                   + ((c%16)/8) * RB*16 + (R%RB) * 16 + (c%8) * 2
// with KS = n_pad/16 and zero fill past rows / cols; row_shift (optional)
// is subtracted from every element of its row first, and `shifted`
// (optional) receives the shifted FP32 matrix in src's own layout.  One thread writes the
// 8 columns of one (row, k-block): 16 bytes hi and 16 bytes lo.
__global__ void tile_split_kernel(const float* __restrict__ src, int64_t ld_src, int transpose, int64_t rows,
                                  int cols, const float* __restrict__ row_shift, int rb, int ks_count,
                                  int64_t n_blk, __nv_bfloat16* __restrict__ dst, float* __restrict__ shifted) {
  const int64_t total = n_blk * ks_count * 2 * rb;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int r = static_cast<int>(idx % rb);
    int64_t rest = idx / rb;
    const int kb = static_cast<int>(rest % 2);
    rest /= 2;
    const int ks = static_cast<int>(rest % ks_count);
    const int64_t blk = rest / ks_count;
    const int64_t R = blk * rb + r;
    const int c0 = ks * kTcK + kb * 8;
    const float sh = (row_shift != nullptr && R < rows) ? row_shift[R] : 0.0f;
    __align__(16) __nv_bfloat16 h[8];
    __align__(16) __nv_bfloat16 l[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int c = c0 + e;
      float x = 0.0f;
      if (R < rows && c < cols) {
        const int64_t at = transpose ? (int64_t)c * ld_src + R : R * ld_src + c;
        x = src[at] - sh;
        if (shifted != nullptr) shifted[at] = x;  // the shifted FP32 matrix, same layout as src
      }
      h[e] = __float2bfloat16_rn(x);
      l[e] = __float2bfloat16_rn(x - __bfloat162float(h[e]));
    }
    const int64_t base = ((blk * ks_count + ks) * 2) * (int64_t)rb * kTcK + (int64_t)kb * rb * 8 + (int64_t)r * 8;
    *reinterpret_cast<uint4*>(dst + base) = *reinterpret_cast<const uint4*>(h);
    *reinterpret_cast<uint4*>(dst + base + (int64_t)rb * kTcK) = *reinterpret_cast<const uint4*>(l);
  }
}

// Per-column mean of Y [n][ldy] (the per-vertex centre of the data): FP32
// sums of 16-row blocks accumulated in FP64 (the centre only has to be close
// to the mean -- the GLM restores the betas with the same value -- and FP64
// adds are scarce on this part).
__global__ void col_mean_kernel(const float* __restrict__ Y, int64_t ldy, int n, int64_t V, float* __restrict__ mean) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int i0 = 0; i0 < n; i0 += 16) {
      float b = 0.0f;
      const int i1 = min(n, i0 + 16);
      for (int i = i0; i < i1; ++i) b += __ldg(Y + (int64_t)i * ldy + v);
      s += static_cast<double>(b);
    }
    mean[v] = static_cast<float>(s / n);
  }
}

// out = Y minus each column's centre (the data centred per vertex).
__global__ void col_center_kernel(const float* __restrict__ Y, int64_t ldy, int n, int64_t V,
                                  const float* __restrict__ centre, float* __restrict__ out) {
  const int64_t total = (int64_t)n * V;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / V, v = e % V;
    out[i * ldy + v] = Y[i * ldy + v] - centre[v];
  }
}

// Centred sum of squares of every column of Yc [n][ldy] (the data minus its
// per-vertex centre): sum (y - m)^2 with m the column's mean, as
// S2 - S1^2 / n from FP32 sums of 16-row blocks accumulated in FP64.
__global__ void col_sumsq_kernel(const float* __restrict__ Yc, int64_t ldy, int n, int64_t V,
                                 float* __restrict__ yy) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    double s1 = 0.0, s2 = 0.0;
    for (int i0 = 0; i0 < n; i0 += 16) {
      float b1 = 0.0f, b2 = 0.0f;
      const int i1 = min(n, i0 + 16);
      for (int i = i0; i < i1; ++i) {
        const float x = __ldg(Yc + (int64_t)i * ldy + v);
        b1 += x;
        b2 = fmaf(x, x, b2);
      }
      s1 += static_cast<double>(b1);
      s2 += static_cast<double>(b2);
    }
    yy[v] = static_cast<float>(fmax(s2 - s1 * s1 / n, 0.0));
  }
}

// --- the GEMM + residual epilogue -----------------------------------------------
struct TcArgs {
  const __nv_bfloat16* yt;  // pre-tiled data, 128-vertex row blocks
  const __nv_bfloat16* pt;  // pre-tiled pseudoinverse rows, DB*8-row blocks
  const float* xt;          // [n_db][n_sc][kmax][DB] negated design rows (zero padded)
  const float* Y;           // FP32 data [n][ldy]
  const float* Yc;          // data minus its per-vertex centre (or null): with it every design has an
                            // intercept and its rows come centred, so residuals skip the intercept term
  const float* shift;       // per-vertex centre subtracted before the split (or null)
  const float* u;           // [G_pad][kmax] pinv(X_d).1 (with shift)
  const float* invdiag;     // [G][kmax]
  const float* dof;         // [G]
  const int32_t* coef;      // mode 0: coefficient indices; mode 2: (start, width) per column group;
                            // mode 3: (kind, column, width, weight offset) per output row
  const float* wmat;        // modes 2, 3: [G][w_stride] per-design weights (blocks of inv(X'X))
  float* t_out;             // [G][n_coef][ldt]
  int64_t ldy, ldt, V;
  int32_t n, n_sc, ks_count, G, n_db, n_coef, mode, w_stride;
  int32_t* err;
};

// Tensor memory for N accumulator columns (warp 0) and the pipeline's
// barriers (thread 0: full[4], empty[4], done); returns the TMEM address.
// Every thread of the CTA calls it (it synchronises the CTA).
template <int N>
__device__ __forceinline__ uint32_t tc_setup(uint32_t* sTmem, uint32_t full0, uint32_t empty0, uint32_t done,
                                             int* sFail, int warp, int tid) {
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(sTmem)),
                 "n"(N)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < kTcStages; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    mbar_init(done, 1);
    *sFail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  return *sTmem;
}

// ---- copy / MMA pipeline, run by one thread ----
// K steps of D[128][N] += A . B over the pre-tiled operands: a 4-stage ring of
// one cp.async.bulk per operand per stage (completing on the stage's full
// barrier); the three split products of a step are committed to the stage's
// empty barrier, and a stage is refilled one step behind the MMA issue.
// Commits `done` after the last step.  On a wait that ran out: records
// kDevLoopLimit, sets *sFail and waits (bounded) for the copies in flight.
template <int N>
__device__ __forceinline__ void tc_gemm_pipeline(const unsigned char* ysrc, const unsigned char* psrc,
                                                 uint32_t sbase, uint32_t full0, uint32_t empty0, uint32_t done,
                                                 uint32_t tmem, int KS, int32_t* err, int* sFail) {
  constexpr int YS = tc_y_stage();
  constexpr int PS = N * kTcK * 2 * 2;
  constexpr int ST = YS + PS;
  const uint32_t idesc = make_idesc(kTcM, N);
  int issued = 0;  // K steps whose copies were issued
  bool ok = true;
  for (; issued < kTcStages && issued < KS; ++issued) {
    const uint32_t dst = sbase + issued * ST, fb = full0 + 8 * issued;
    mbar_expect_tx(fb, YS + PS);
    bulk_g2s(dst, ysrc + (int64_t)issued * YS, YS, fb);
    bulk_g2s(dst + YS, psrc + (int64_t)issued * PS, PS, fb);
  }
  int ks = 0;  // K steps whose copies were consumed
  for (; ks < KS; ++ks) {
    const int s = ks % kTcStages;
    if (!mbar_wait(full0 + 8 * s, (ks / kTcStages) & 1)) {
      ok = false;
      break;
    }
    tc_fence_after();
    const uint32_t st = sbase + s * ST;
    const uint64_t ah = make_desc(st, kTcM * 16, 128);
    const uint64_t al = make_desc(st + YS / 2, kTcM * 16, 128);
    const uint64_t bh = make_desc(st + YS, N * 16, 128);
    const uint64_t bl = make_desc(st + YS + PS / 2, N * 16, 128);
    mma_bf16(tmem, ah, bh, idesc, ks > 0 ? 1u : 0u);
    mma_bf16(tmem, ah, bl, idesc, 1u);
    mma_bf16(tmem, al, bh, idesc, 1u);
    mma_commit(empty0 + 8 * s);
    // refill the stage of step ks-1 (its MMAs are queued ahead of this step's)
    if (ks >= 1 && issued < KS) {
      const int kp = ks - 1, sp = kp % kTcStages;
      if (!mbar_wait(empty0 + 8 * sp, (kp / kTcStages) & 1)) {
        ok = false;
        ++ks;
        break;
      }
      const uint32_t dst = sbase + sp * ST, fb = full0 + 8 * sp;
      mbar_expect_tx(fb, YS + PS);
      bulk_g2s(dst, ysrc + (int64_t)issued * YS, YS, fb);
      bulk_g2s(dst + YS, psrc + (int64_t)issued * PS, PS, fb);
      ++issued;
    }
  }
  mma_commit(done);
  if (!ok) {
    atomicCAS(err, 0, kDevLoopLimit);
    *sFail = 1;
    // copies issued but not consumed: wait (bounded) until they have landed
    for (int qq = ks; qq < issued; ++qq) mbar_wait(full0 + 8 * (qq % kTcStages), (qq / kTcStages) & 1);
  }
}

template <int KMAX, bool kCentred, int DPT_ = tc_dpt(KMAX)>
__global__ void __launch_bounds__(kTcThreads, 2) glm_tc_kernel(TcArgs a) {
  // centred form: r = (y - c) - Xc b[1..] for designs with an intercept
  // (column means removed from the other columns; c the data's centre)
  constexpr int J0 = kCentred ? 1 : 0;
  constexpr int DPT = DPT_;
  constexpr int DB = tc_db(DPT);
  constexpr int N = tc_n(DPT);
  constexpr int YS = tc_y_stage();
  constexpr int PS = tc_p_stage(DPT);
  constexpr int XC = tc_xchunk(KMAX, DPT);
  extern __shared__ __align__(1024) unsigned char sm[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + tc_area(KMAX, DPT));  // full[4], empty[4], done
  uint32_t* sTmem = reinterpret_cast<uint32_t*>(bars + 2 * kTcStages + 1);
  int* sFail = reinterpret_cast<int*>(sTmem + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t vb = blockIdx.x / a.n_db;
  const int db = static_cast<int>(blockIdx.x % a.n_db);
  const uint32_t sbase = smem_addr(sm);
  const uint32_t full0 = smem_addr(bars), empty0 = full0 + 8 * kTcStages, done = full0 + 16 * kTcStages;

  const uint32_t tmem = tc_setup<N>(sTmem, full0, empty0, done, sFail, warp, tid);
  const int KS = a.ks_count;

  // ---- copy / MMA pipeline (one thread) ----
  // the producer thread alone waits for the accumulator; the other warps
  // wait at the CTA barrier (no issue slots spent polling)
  if (tid == 0) {
    tc_gemm_pipeline<N>(reinterpret_cast<const unsigned char*>(a.yt) + (vb * KS) * (int64_t)YS,
                        reinterpret_cast<const unsigned char*>(a.pt) + ((int64_t)db * KS) * (int64_t)PS, sbase,
                        full0, empty0, done, tmem, KS, a.err, sFail);
    if (!mbar_wait(done, 0)) {
      atomicCAS(a.err, 0, kDevLoopLimit);
      *sFail = 1;
    }
    fence_proxy_async();
    tc_fence_before();
  }
  __syncthreads();
  tc_fence_after();
  fence_proxy_async();
  const bool failed = *sFail != 0;

  // ---- drain: TMEM lane = vertex -> sB[(d*KMAX + j)*kTcBld + vertex] ----
  float* sB = reinterpret_cast<float*>(sm);
  if (!failed) {
    const int q = warp & 3, half = warp >> 2;
    const int vl = q * 32 + lane;
#pragma unroll
    for (int dd = 0; dd < DPT; ++dd) {
      float t8[8];
      tmem_ld8(tmem + (static_cast<uint32_t>(q * 32) << 16) + (half * DPT + dd) * kTcRowsPerDesign, t8);
#pragma unroll
      for (int j = 0; j < KMAX; ++j) sB[((half * DPT + dd) * KMAX + j) * kTcBld + vl] = t8[j];
    }
  }
  tc_fence_before();
  __syncthreads();

  // ---- residual pass: lane = design d, thread = VT consecutive vertices ----
  constexpr int VT = DB / 2;
  constexpr int YC = tc_ychunk();
  static_assert((kTcThreads / DB) * VT == kTcM, "threads cover the tile");
  const int d = tid % DB, vg = tid / DB;
  const int g = db * DB + d;
  const int vl0 = vg * VT;
  const int64_t v0 = vb * kTcM + vl0;
  float2 bp[VT / 2][KMAX];
  float2 rss[VT / 2];
  {
    float u[KMAX];
#pragma unroll
    for (int j = 0; j < KMAX; ++j) u[j] = (a.shift != nullptr) ? __ldg(a.u + g * KMAX + j) : 0.0f;
#pragma unroll
    for (int vv = 0; vv < VT; ++vv) {
      const float m = (a.shift != nullptr && v0 + vv < a.V) ? __ldg(a.shift + v0 + vv) : 0.0f;
#pragma unroll
      for (int j = 0; j < KMAX; ++j) {
        const float bv = (failed || j < J0) ? 0.0f : fmaf(m, u[j], sB[(d * KMAX + j) * kTcBld + vl0 + vv]);
        if (vv & 1) bp[vv / 2][j].y = bv; else bp[vv / 2][j].x = bv;
      }
    }
#pragma unroll
    for (int p = 0; p < VT / 2; ++p) rss[p] = make_float2(0.0f, 0.0f);
  }
  __syncthreads();  // the beta area becomes the chunk buffers

  const int n_chunks = a.n_sc / kTcSubjChunk;
  const float* xsrc = a.xt != nullptr ? a.xt + (int64_t)db * a.n_sc * KMAX * DB : nullptr;
  const int64_t vt0 = vb * kTcM;
  auto load_chunk = [&](int c) {
    const uint32_t dst = sbase + (c & 1) * (XC + YC);
    const float* src = xsrc + (int64_t)c * kTcSubjChunk * KMAX * DB;
    for (int i = tid; i < XC / 16; i += kTcThreads) cp_async16(dst + i * 16, src + i * 4);
    for (int e = tid; e < kTcSubjChunk * kTcM; e += kTcThreads) {
      const int i = c * kTcSubjChunk + e / kTcM;
      const int64_t v = vt0 + e % kTcM;
      const bool ok = i < a.n && v < a.V;
      const float* ysrc = kCentred ? a.Yc : a.Y;
      cp_async4(dst + XC + e * 4, ok ? ysrc + (int64_t)i * a.ldy + v : ysrc, ok ? 4u : 0u);
    }
    cp_async_commit();
  };
  if (!failed) {
    // mode 4 needs no residuals: its rows are quadratic forms of the betas
    for (int c = 0; a.mode != 4 && c < n_chunks; ++c) {
      if (c == 0) load_chunk(0);
      // chunk c+1 streams into the other buffer while chunk c is used
      if (c + 1 < n_chunks) {
        load_chunk(c + 1);
        cp_async_wait<1>();
      } else {
        cp_async_wait<0>();
      }
      __syncthreads();
      const float* xs = reinterpret_cast<const float*>(sm + (c & 1) * (XC + YC));
      const float* ys = xs + XC / 4;
#pragma unroll 2
      for (int ii = 0; ii < kTcSubjChunk; ++ii) {
        float2 xj[KMAX];
#pragma unroll
        for (int j = J0; j < KMAX; ++j) {
          const float x = xs[(ii * KMAX + j) * DB + d];
          xj[j] = make_float2(x, x);
        }
        const float4* yr = reinterpret_cast<const float4*>(ys + ii * kTcM + vl0);
#pragma unroll
        for (int q4 = 0; q4 < VT / 4; ++q4) {
          const float4 yv = yr[q4];
          float2 r0 = make_float2(yv.x, yv.y), r1 = make_float2(yv.z, yv.w);
#pragma unroll
          for (int j = J0; j < KMAX; ++j) {
            r0 = __ffma2_rn(xj[j], bp[2 * q4][j], r0);
            r1 = __ffma2_rn(xj[j], bp[2 * q4 + 1][j], r1);
          }
          rss[2 * q4] = __ffma2_rn(r0, r0, rss[2 * q4]);
          rss[2 * q4 + 1] = __ffma2_rn(r1, r1, rss[2 * q4 + 1]);
        }
      }
      __syncthreads();
    }
    if (g < a.G && a.mode == 0) {
      // t of each requested coefficient
      const float inv_dof = 1.0f / __ldg(a.dof + g);
      for (int ci = 0; ci < a.n_coef; ++ci) {
        const int j = __ldg(a.coef + ci);
        const float dj = __ldg(a.invdiag + g * KMAX + j);
        float* dst = a.t_out + ((int64_t)g * a.n_coef + ci) * a.ldt + v0;
#pragma unroll
        for (int vv = 0; vv < VT; ++vv) {
          if (v0 + vv < a.V) {
            float bj = 0.0f;
#pragma unroll
            for (int jj = J0; jj < KMAX; ++jj)
              if (jj == j) bj = (vv & 1) ? bp[vv / 2][jj].y : bp[vv / 2][jj].x;
            const float rs = (vv & 1) ? rss[vv / 2].y : rss[vv / 2].x;
            dst[vv] = bj / sqrtf(rs * inv_dof * dj);
          }
        }
      }
    } else if (g < a.G && a.mode == 1) {
      // residual sum of squares (from the residuals)
      float* dst = a.t_out + (int64_t)g * a.ldt + v0;
#pragma unroll
      for (int vv = 0; vv < VT; ++vv)
        if (v0 + vv < a.V) dst[vv] = (vv & 1) ? rss[vv / 2].y : rss[vv / 2].x;
    } else if (g < a.G && a.mode >= 2) {
      // mode 2: partial F of each column group; mode 3: a program of typed
      // output rows (t, -t, partial F, cosinor amplitude / acrophase t, extra
      // sum of squares); mode 4: a program of extra-sum-of-squares rows only,
      // without the residual pass.
      // this thread's betas and RSS go to its own slice of the (now free)
      // shared area, so the output loops index them at run time
      float* mine = reinterpret_cast<float*>(sm) + tid * VT * (KMAX + 1);
#pragma unroll
      for (int vv = 0; vv < VT; ++vv) {
#pragma unroll
        for (int jj = 0; jj < KMAX; ++jj)
          mine[vv * (KMAX + 1) + jj] = (jj < J0) ? 0.0f : ((vv & 1) ? bp[vv / 2][jj].y : bp[vv / 2][jj].x);
        mine[vv * (KMAX + 1) + KMAX] = (vv & 1) ? rss[vv / 2].y : rss[vv / 2].x;
      }
      const float dof = a.dof != nullptr ? __ldg(a.dof + g) : 1.0f;
      const float inv_dof = 1.0f / dof;
      const float* wg = a.wmat + (int64_t)g * a.w_stride;
      int woff = 0;
      for (int oi = 0; oi < a.n_coef; ++oi) {
        int kind, j, kv, wo;
        if (a.mode == 2) {
          kind = kTcOutF;
          j = __ldg(a.coef + 2 * oi);
          kv = __ldg(a.coef + 2 * oi + 1);
          wo = woff;
          woff += (kv >= 1 && kv <= KMAX) ? kv * kv : 0;
        } else {
          kind = __ldg(a.coef + 4 * oi);
          j = __ldg(a.coef + 4 * oi + 1);
          kv = __ldg(a.coef + 4 * oi + 2);
          wo = __ldg(a.coef + 4 * oi + 3);
        }
        bool ok;
        if (a.mode == 4 && kind != kTcOutEss) {
          ok = false;  // no residual sum of squares in this mode
        } else if (kind == kTcOutT || kind == kTcOutNegT) {
          ok = j >= 0 && j < KMAX;
        } else if (kind == kTcOutF || kind == kTcOutEss) {
          // written without sums that could overflow on a corrupt program row
          ok = j >= 0 && j < KMAX && kv >= 1 && kv <= KMAX - j && wo >= 0 && wo <= a.w_stride - kv * kv;
        } else if (kind == kTcOutAmp || kind == kTcOutAcro) {
          ok = j >= 0 && j < KMAX - 1 && wo >= 0 && wo <= a.w_stride - 3;
        } else {
          ok = false;
        }
        const float dj = (ok && kind <= kTcOutNegT) ? __ldg(a.invdiag + g * KMAX + j) : 0.0f;
        float* dst = a.t_out + ((int64_t)g * a.n_coef + oi) * a.ldt + v0;
        for (int vv = 0; vv < VT; ++vv) {
          if (v0 + vv >= a.V) break;
          const float* bv = mine + vv * (KMAX + 1);
          const float rs = bv[KMAX];
          float val = __int_as_float(0x7fc00000);
          if (!ok) {
          } else if (kind == kTcOutT || kind == kTcOutNegT) {
            val = bv[j] / sqrtf(rs * inv_dof * dj);
            if (kind == kTcOutNegT) val = -val;
          } else if (kind == kTcOutF || kind == kTcOutEss) {
            // the extra sum of squares of dropping S, RSS_without_S - RSS, in
            // its exact Wald form b_S' inv(inv(X'X)_SS) b_S -- no difference of
            // two residual sums; F: divided by |S| and RSS / dof
            float q = 0.0f;
            for (int ja = 0; ja < kv; ++ja)
              for (int jc = 0; jc < kv; ++jc)
                q = fmaf(bv[j + ja] * __ldg(wg + wo + ja * kv + jc), bv[j + jc], q);
            val = (kind == kTcOutEss) ? q : (q / static_cast<float>(kv)) / (rs / dof);
          } else {
            // cosinor pair (b1, b2) = (cos, sin) coefficients, wg = inv(X'X)
            // entries (11, 12, 22): with A^2 = b1^2 + b2^2 and the acrophase
            // angle's |sin| = |b2|/A, |cos| = |b1|/A,
            //   t_amplitude = A^2 / (sigma sqrt(I11 b1^2 - 2 I12 |b1 b2| + I22 b2^2))
            //   t_acrophase = A^2 / (sigma sqrt(I11 b2^2 + 2 I12 |b1 b2| + I22 b1^2))
            const float b1 = bv[j], b2 = bv[j + 1];
            const float i11 = __ldg(wg + wo), i12 = __ldg(wg + wo + 1), i22 = __ldg(wg + wo + 2);
            const float a2 = fmaf(b1, b1, b2 * b2);
            const float c = 2.0f * i12 * fabsf(b1 * b2);
            const float q = (kind == kTcOutAmp) ? fmaf(i11, b1 * b1, fmaf(i22, b2 * b2, -c))
                                                : fmaf(i11, b2 * b2, fmaf(i22, b1 * b1, c));
            val = a2 / sqrtf(rs * inv_dof * q);
          }
          dst[vv] = val;
        }
      }
    }
  }
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(N) : "memory");
  }
}


// --- the quadratic-form GLM (centred designs, t of coefficients >= 1) ---------
// For designs whose first column is all ones, and t of the other coefficients
// only (the permutation engines' case), everything follows from the cross
// products of the centred design columns with the centred data,
// c_d(v) = Xc_d' (y(v) - centre(v)), by Frisch-Waugh (the intercept drops out):
//   b   = inv(Xc'Xc) c                         the betas of columns 1..k-1
//   RSS = yy - c'b, yy = sum_i (y_i - mean)^2  the residual sum of squares
//   t_j = b_j / sqrt(RSS / dof * inv(X'X)_jj)  (cynumstats.pyx:47-64)
// One GEMM D[v][d*R + j] = sum_i (y_i(v) - centre(v)) Xc_d[i][j] -- R = 4 rows
// per design for k <= 5 (64 designs per 256-column tile), 8 for k <= 8 (32)
// -- and an epilogue of O(k^2) FMAs per (vertex, design) replace the
// residual pass's (k+1) n.  RSS = yy - c'b is first-order in the split error
// of c, scaled by R^2 / (1 - R^2) of the fit; the split error of a cross
// product is a sum of independent roundings while the product itself is
// coherent, so at the fits a permutation null produces (R^2 ~ k / n) the t
// error stays that of the betas.
constexpr int kQfN = 256;       // accumulator columns (MMA N)
constexpr int kQfMaxCoef = 8;   // coefficients per design
__host__ __device__ constexpr int qf_rows(int kc) { return kc <= 4 ? 4 : 8; }  // B rows per design
__host__ __device__ constexpr int qf_db(int kc) { return kQfN / qf_rows(kc); }  // designs per tile
__host__ __device__ constexpr int qf_stage() { return tc_y_stage() + kQfN * kTcK * 2 * 2; }
__host__ __device__ constexpr int qf_smem() { return kTcStages * qf_stage() + 128; }
static_assert(qf_smem() <= 113 * 1024, "two CTAs per SM");

struct QfArgs {
  const __nv_bfloat16* yt;  // pre-tiled centred data, 128-vertex row blocks
  const __nv_bfloat16* xt;  // pre-tiled centred design columns, R rows per design, 256-row blocks
  const float* yy;          // [V] centred sum of squares of each vertex's data
  const float* ginv;        // [G_pad][R][R] inv(Xc'Xc) = inv(X'X) without its first row and column, zero padded
  const float* invdiag;     // [G][KC + 1] SE factors
  const float* dof;         // [G]
  const int32_t* coef;      // coefficient indices in [1, KC]
  float* t_out;             // [G][n_coef][ldt]
  int64_t ldt, V;
  int32_t ks_count, G, n_db, n_coef;
  int32_t* err;
};

// The quadratic-form epilogue of one warp: the DB/2 designs of the tile from
// design `dfirst` on (global index gbase + dfirst + ...), read from the TMEM
// accumulator columns at `tacc` (lane quarter included) for vertex v of this
// lane.  Every lane works on the same design at a time, so the per-design
// constants are warp-uniform loads and the t stores coalesce over the vertices.
template <int KC>
__device__ __forceinline__ void qf_epilogue_warp(const QfArgs& a, uint32_t tacc, int dfirst, int gbase, int64_t v) {
  constexpr int R = qf_rows(KC), DB = qf_db(KC);
  const bool live = v < a.V;
  const float yyv = live ? __ldg(a.yy + v) : 0.0f;
  int jc[kQfMaxCoef];  // the requested coefficients (uniform)
#pragma unroll
  for (int ci = 0; ci < kQfMaxCoef; ++ci) jc[ci] = (ci < a.n_coef) ? __ldg(a.coef + ci) : 0;
  constexpr int DPW = DB / 2;  // designs per warp
  constexpr int DPL = 16 / R;  // designs per 16-column load
#pragma unroll 1
  for (int d0 = 0; d0 < DPW; d0 += DPL) {
    float cc[16];
    tmem_ld16(tacc + d0 * R, cc);
#pragma unroll
    for (int dd = 0; dd < DPL; ++dd) {
      const int g = gbase + dfirst + d0 + dd;
      if (g >= a.G) break;
      // b = inv(Xc'Xc) c from the padded R x R inverse, rows as float4
      const float4* gi = reinterpret_cast<const float4*>(a.ginv + (int64_t)g * R * R);
      float b[KC];
      float qf = 0.0f;
#pragma unroll
      for (int i = 0; i < KC; ++i) {
        float row[R];
#pragma unroll
        for (int r4 = 0; r4 < (KC + 3) / 4; ++r4) {
          const float4 x4 = __ldg(gi + i * (R / 4) + r4);
          row[4 * r4] = x4.x;
          row[4 * r4 + 1] = x4.y;
          row[4 * r4 + 2] = x4.z;
          row[4 * r4 + 3] = x4.w;
        }
        float s = 0.0f;
#pragma unroll
        for (int j = 0; j < KC; ++j) s = fmaf(row[j], cc[dd * R + j], s);
        b[i] = s;
        qf = fmaf(cc[dd * R + i], s, qf);
      }
      // sigma^2 = RSS / dof; t_j = b_j / sqrt(sigma^2 inv(X'X)_jj)
      const float s2 = fmaxf(yyv - qf, 0.0f) / __ldg(a.dof + g);
#pragma unroll
      for (int ci = 0; ci < kQfMaxCoef; ++ci) {
        if (ci >= a.n_coef) break;
        const int j = jc[ci];
        float bj = __int_as_float(0x7fc00000);  // NaN for a coefficient outside [1, KC]
#pragma unroll
        for (int jj = 0; jj < KC; ++jj)
          if (jj + 1 == j) bj = b[jj];
        const float dj = (j >= 1 && j <= KC) ? __ldg(a.invdiag + (int64_t)g * (KC + 1) + j) : 1.0f;
        if (live) a.t_out[((int64_t)g * a.n_coef + ci) * a.ldt + v] = bj * rsqrtf(s2 * dj);
      }
    }
  }
}

template <int KC>
__global__ void __launch_bounds__(kTcThreads, 2) glm_tc_qf_kernel(QfArgs a) {
  constexpr int R = qf_rows(KC), DB = qf_db(KC), N = kQfN;
  constexpr int YS = tc_y_stage(), PS = N * kTcK * 2 * 2;
  extern __shared__ __align__(1024) unsigned char sm[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + kTcStages * qf_stage());  // full[4], empty[4], done
  uint32_t* sTmem = reinterpret_cast<uint32_t*>(bars + 2 * kTcStages + 1);
  int* sFail = reinterpret_cast<int*>(sTmem + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t vb = blockIdx.x / a.n_db;
  const int db = static_cast<int>(blockIdx.x % a.n_db);
  const uint32_t sbase = smem_addr(sm);
  const uint32_t full0 = smem_addr(bars), empty0 = full0 + 8 * kTcStages, done = full0 + 16 * kTcStages;
  const uint32_t tmem = tc_setup<N>(sTmem, full0, empty0, done, sFail, warp, tid);
  const int KS = a.ks_count;

  // the producer thread alone waits for the accumulator; the other warps
  // wait at the CTA barrier (no issue slots spent polling)
  if (tid == 0) {
    tc_gemm_pipeline<N>(reinterpret_cast<const unsigned char*>(a.yt) + (vb * KS) * (int64_t)YS,
                        reinterpret_cast<const unsigned char*>(a.xt) + ((int64_t)db * KS) * (int64_t)PS, sbase,
                        full0, empty0, done, tmem, KS, a.err, sFail);
    if (!mbar_wait(done, 0)) {
      atomicCAS(a.err, 0, kDevLoopLimit);
      *sFail = 1;
    }
    tc_fence_before();
  }
  __syncthreads();
  tc_fence_after();

  if (*sFail == 0) {
    const int q = warp & 3, half = warp >> 2;
    qf_epilogue_warp<KC>(a, tmem + (static_cast<uint32_t>(q * 32) << 16) + half * (DB / 2) * R, half * (DB / 2),
                         db * DB, vb * kTcM + q * 32 + lane);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(N) : "memory");
  }
}

template <int KC>
static int launch_tc_qf(const QfArgs& a, int64_t n_vb, cudaStream_t stream) {
  const int smem = qf_smem();
  TFGB_CUDA(cudaFuncSetAttribute(glm_tc_qf_kernel<KC>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  glm_tc_qf_kernel<KC><<<static_cast<unsigned>(n_vb * a.n_db), kTcThreads, smem, stream>>>(a);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

template <int KMAX, int DPT = tc_dpt(KMAX)>
static int launch_tc(const TcArgs& a, int64_t n_vb, cudaStream_t stream) {
  const int smem = tc_smem(KMAX, DPT);
  const int64_t grid = n_vb * a.n_db;
  if (a.Yc != nullptr) {
    TFGB_CUDA(cudaFuncSetAttribute(glm_tc_kernel<KMAX, true, DPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   smem));
    glm_tc_kernel<KMAX, true, DPT><<<static_cast<unsigned>(grid), kTcThreads, smem, stream>>>(a);
  } else {
    TFGB_CUDA(cudaFuncSetAttribute(glm_tc_kernel<KMAX, false, DPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   smem));
    glm_tc_kernel<KMAX, false, DPT><<<static_cast<unsigned>(grid), kTcThreads, smem, stream>>>(a);
  }
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

}  // namespace tfgb

extern "C" {

int glm_tc_design_block(int32_t kmax) {
  if (kmax < 1 || kmax > tfgb::kTcRowsPerDesign) return -1;
  return tfgb::tc_db(tfgb::tc_dpt(kmax));
}

int glm_qf_design_block(int32_t kmax) {
  if (kmax < 2 || kmax > tfgb::kTcRowsPerDesign) return -1;
  return tfgb::qf_db(kmax - 1);
}

int glm_col_sumsq(const float* Y_centred, int64_t ldy, int32_t n, int64_t V, float* yy, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(Y_centred && yy, "NULL pointer");
  TFGB_CHECK_ARG(n > 0 && V >= 0 && ldy >= V, "bad sizes");
  if (V == 0) return TFCE_OK;
  const unsigned blocks = static_cast<unsigned>(std::min<int64_t>((V + 255) / 256, 152 * 16));
  tfgb::col_sumsq_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(Y_centred, ldy, n, V, yy);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

int glm_tstat_tc_qf(const void* y_tiles, const float* yy, int32_t n, int32_t n_pad, int64_t V,
                    const void* x_tiles, const float* ginv, const float* invdiag, const float* dof, int32_t G,
                    int32_t kmax, const int32_t* coef, int32_t n_coef, float* t_out, int64_t ldt, int32_t* err,
                    void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(y_tiles && yy && x_tiles && ginv && invdiag && dof && coef && t_out && err, "NULL pointer");
  TFGB_CHECK_ARG(kmax >= 2 && kmax <= tfgb::kTcRowsPerDesign, "kmax must be in [2, 8]");
  TFGB_CHECK_ARG(n > kmax && n_pad >= n && n_pad % tfgb::kTcK == 0, "n_pad must be >= n and a multiple of 16");
  TFGB_CHECK_ARG(n_coef >= 1 && n_coef <= tfgb::kQfMaxCoef, "n_coef must be in [1, 8]");
  TFGB_CHECK_ARG(V >= 0 && G >= 0 && ldt >= V, "bad sizes");
  TFGB_CHECK_ARG(reinterpret_cast<uintptr_t>(y_tiles) % 16 == 0 && reinterpret_cast<uintptr_t>(x_tiles) % 16 == 0 &&
                     reinterpret_cast<uintptr_t>(ginv) % 16 == 0,
                 "tiles and ginv must be 16-byte aligned");
  if (V == 0 || G == 0) return TFCE_OK;
  tfgb::QfArgs a{};
  a.yt = static_cast<const __nv_bfloat16*>(y_tiles);
  a.xt = static_cast<const __nv_bfloat16*>(x_tiles);
  a.yy = yy;
  a.ginv = ginv;
  a.invdiag = invdiag;
  a.dof = dof;
  a.coef = coef;
  a.t_out = t_out;
  a.ldt = ldt;
  a.V = V;
  a.ks_count = n_pad / tfgb::kTcK;
  a.G = G;
  a.n_db = (G + glm_qf_design_block(kmax) - 1) / glm_qf_design_block(kmax);
  a.n_coef = n_coef;
  a.err = err;
  const int64_t n_vb = (V + tfgb::kTcM - 1) / tfgb::kTcM;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  switch (kmax - 1) {
    case 1: return tfgb::launch_tc_qf<1>(a, n_vb, st);
    case 2: return tfgb::launch_tc_qf<2>(a, n_vb, st);
    case 3: return tfgb::launch_tc_qf<3>(a, n_vb, st);
    case 4: return tfgb::launch_tc_qf<4>(a, n_vb, st);
    case 5: return tfgb::launch_tc_qf<5>(a, n_vb, st);
    case 6: return tfgb::launch_tc_qf<6>(a, n_vb, st);
    default: return tfgb::launch_tc_qf<7>(a, n_vb, st);
  }
}

int64_t glm_tile_bytes(int64_t rows, int32_t row_block, int32_t n_pad) {
  if (rows < 0 || row_block <= 0 || n_pad <= 0 || n_pad % tfgb::kTcK) return -1;
  const int64_t blocks = (rows + row_block - 1) / row_block;
  return blocks * row_block * (int64_t)n_pad * 4;  // hi + lo, 2 bytes each
}

int glm_col_mean(const float* Y, int64_t ldy, int32_t n, int64_t V, float* mean, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(Y && mean, "NULL pointer");
  TFGB_CHECK_ARG(n > 0 && V >= 0 && ldy >= V, "bad sizes");
  if (V == 0) return TFCE_OK;
  const unsigned blocks = static_cast<unsigned>(std::min<int64_t>((V + 255) / 256, 152 * 16));
  tfgb::col_mean_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(Y, ldy, n, V, mean);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

int glm_col_center(const float* Y, int64_t ldy, int32_t n, int64_t V, const float* centre, float* out,
                   void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(Y && centre && out, "NULL pointer");
  TFGB_CHECK_ARG(n > 0 && V >= 0 && ldy >= V, "bad sizes");
  if (V == 0) return TFCE_OK;
  const int64_t total = (int64_t)n * V;
  const unsigned blocks = static_cast<unsigned>(std::min<int64_t>((total + 255) / 256, 152 * 32));
  tfgb::col_center_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(Y, ldy, n, V, centre, out);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

int glm_tile_split(const float* src, int64_t ld_src, int32_t transpose, int64_t rows, int32_t cols,
                   const float* row_shift, int32_t row_block, int32_t n_pad, void* dst, float* shifted, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(src && dst, "NULL pointer");
  TFGB_CHECK_ARG(rows >= 0 && cols >= 0 && n_pad >= cols && n_pad % tfgb::kTcK == 0,
                 "n_pad must be >= cols and a multiple of 16");
  TFGB_CHECK_ARG(row_block > 0 && row_block % 8 == 0 && row_block <= 256,
                 "row_block must be a multiple of 8 in [8, 256]");
  if (rows == 0) return TFCE_OK;
  const int64_t n_blk = (rows + row_block - 1) / row_block;
  const int ks = n_pad / tfgb::kTcK;
  const int64_t total = n_blk * ks * 2 * row_block;
  const unsigned blocks = static_cast<unsigned>(std::min<int64_t>((total + 255) / 256, 152 * 16));
  tfgb::tile_split_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      src, ld_src, transpose, rows, cols, row_shift, row_block, ks, n_blk, static_cast<__nv_bfloat16*>(dst), shifted);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

int glm_stat_tc_block(const void* y_tiles, const float* y_shift, const float* Y, const float* Y_centred,
                      int64_t ldy, int32_t n, int32_t n_pad, int64_t V, const void* p_tiles, const float* u_rows,
                      const float* x_rows, int32_t n_sc, const float* invdiag, const float* dof, int32_t G,
                      int32_t kmax, int32_t design_block, int32_t mode, const int32_t* coef, int32_t n_coef,
                      const float* wmat, int32_t w_stride, float* t_out, int64_t ldt, int32_t* err, void* stream) {
  tfgb::clear_error();
  if (design_block == 0 && kmax >= 1 && kmax <= tfgb::kTcRowsPerDesign) design_block = glm_tc_design_block(kmax);
  TFGB_CHECK_ARG(design_block == 16 || (design_block == 32 && kmax <= 5),
                 "design_block must be 32 (kmax <= 5) or 16");
  TFGB_CHECK_ARG(y_tiles && Y && p_tiles && t_out && err, "NULL pointer");
  TFGB_CHECK_ARG(mode == 4 || (x_rows && invdiag && dof), "x_rows / invdiag / dof are NULL");
  TFGB_CHECK_ARG(mode == 1 || coef != nullptr, "coef is NULL");
  TFGB_CHECK_ARG(!y_shift || u_rows, "a centred data operand needs u_rows");
  TFGB_CHECK_ARG(n > 0 && n_pad >= n && n_pad % tfgb::kTcK == 0, "n_pad must be >= n and a multiple of 16");
  TFGB_CHECK_ARG(n_sc >= n && n_sc % tfgb::kTcSubjChunk == 0, "n_sc must be >= n and a multiple of 32");
  TFGB_CHECK_ARG(kmax >= 1 && kmax <= tfgb::kTcRowsPerDesign, "kmax must be in [1, 8]");
  TFGB_CHECK_ARG(mode >= 0 && mode <= 4,
                 "mode must be 0 (t), 1 (RSS), 2 (partial F), 3 (program) or 4 (sums-of-squares program)");
  TFGB_CHECK_ARG(mode == 1 || n_coef >= 1, "n_coef must be >= 1");
  TFGB_CHECK_ARG(mode != 2 || (wmat != nullptr && w_stride >= 1), "partial F needs wmat");
  TFGB_CHECK_ARG(mode < 3 || wmat != nullptr || w_stride == 0, "w_stride > 0 needs wmat");
  TFGB_CHECK_ARG(mode != 4 || Y_centred == nullptr, "mode 4 forms no residuals (Y_centred must be NULL)");
  TFGB_CHECK_ARG(V >= 0 && G >= 0 && ldt >= V && ldy >= V, "bad sizes");
  TFGB_CHECK_ARG(reinterpret_cast<uintptr_t>(y_tiles) % 16 == 0 && reinterpret_cast<uintptr_t>(p_tiles) % 16 == 0 &&
                     reinterpret_cast<uintptr_t>(x_rows) % 16 == 0,
                 "tiles and design rows must be 16-byte aligned");
  if (V == 0 || G == 0) return TFCE_OK;
  tfgb::TcArgs a{};
  a.yt = static_cast<const __nv_bfloat16*>(y_tiles);
  a.pt = static_cast<const __nv_bfloat16*>(p_tiles);
  a.xt = x_rows;
  a.Y = Y;
  a.Yc = Y_centred;
  a.shift = y_shift;
  a.u = u_rows;
  a.invdiag = invdiag;
  a.dof = dof;
  a.coef = coef;
  a.wmat = wmat;
  a.t_out = t_out;
  a.ldy = ldy;
  a.ldt = ldt;
  a.V = V;
  a.n = n;
  a.n_sc = n_sc;
  a.ks_count = n_pad / tfgb::kTcK;
  a.G = G;
  a.n_db = (G + design_block - 1) / design_block;
  a.n_coef = (mode == 1) ? 1 : n_coef;
  a.mode = mode;
  a.w_stride = w_stride;
  a.err = err;
  const int64_t n_vb = (V + tfgb::kTcM - 1) / tfgb::kTcM;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool small = (design_block == 16);
  switch (kmax) {
    case 1: return small ? tfgb::launch_tc<1, 8>(a, n_vb, st) : tfgb::launch_tc<1>(a, n_vb, st);
    case 2: return small ? tfgb::launch_tc<2, 8>(a, n_vb, st) : tfgb::launch_tc<2>(a, n_vb, st);
    case 3: return small ? tfgb::launch_tc<3, 8>(a, n_vb, st) : tfgb::launch_tc<3>(a, n_vb, st);
    case 4: return small ? tfgb::launch_tc<4, 8>(a, n_vb, st) : tfgb::launch_tc<4>(a, n_vb, st);
    case 5: return small ? tfgb::launch_tc<5, 8>(a, n_vb, st) : tfgb::launch_tc<5>(a, n_vb, st);
    case 6: return tfgb::launch_tc<6>(a, n_vb, st);
    case 7: return tfgb::launch_tc<7>(a, n_vb, st);
    default: return tfgb::launch_tc<8>(a, n_vb, st);
  }
}

int glm_stat_tc(const void* y_tiles, const float* y_shift, const float* Y, const float* Y_centred, int64_t ldy,
                int32_t n, int32_t n_pad, int64_t V, const void* p_tiles, const float* u_rows, const float* x_rows,
                int32_t n_sc, const float* invdiag, const float* dof, int32_t G, int32_t kmax, int32_t mode,
                const int32_t* coef, int32_t n_coef, const float* wmat, int32_t w_stride, float* t_out,
                int64_t ldt, int32_t* err, void* stream) {
  return glm_stat_tc_block(y_tiles, y_shift, Y, Y_centred, ldy, n, n_pad, V, p_tiles, u_rows, x_rows, n_sc, invdiag,
                           dof, G, kmax, 0, mode, coef, n_coef, wmat, w_stride, t_out, ldt, err, stream);
}

int glm_tstat_tc(const void* y_tiles, const float* y_shift, const float* Y, int64_t ldy, int32_t n,
                 int32_t n_pad, int64_t V, const void* p_tiles, const float* u_rows, const float* x_rows,
                 int32_t n_sc, const float* invdiag, const float* dof, int32_t G, int32_t kmax,
                 const int32_t* coef, int32_t n_coef, float* t_out, int64_t ldt, int32_t* err, void* stream) {
  return glm_stat_tc(y_tiles, y_shift, Y, nullptr, ldy, n, n_pad, V, p_tiles, u_rows, x_rows, n_sc, invdiag, dof, G,
                     kmax, 0, coef, n_coef, nullptr, 0, t_out, ldt, err, stream);
}

}  // extern "C"
