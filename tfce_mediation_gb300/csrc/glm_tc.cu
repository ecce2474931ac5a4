// Tensor-core (tcgen05) form of the permuted-design GLM: the stacked
// pseudoinverses of G designs, P = [G*8][n] (rows of inv(X'X)X', padded to 8
// rows per design), times the data Y [n][V], as one GEMM per 64-vertex tile
// with an FP32 accumulator in tensor memory, followed by the residual / RSS /
// SE / t epilogue on the CUDA cores (cynumstats.pyx:28-29, 47-64: RSS from the
// residuals y - X.beta, never from Y'Y).
//
// Precision: split BF16 -- every operand is stored as hi = bf16(x) and
// lo = bf16(x - hi), and beta = P_hi.Y_hi + P_hi.Y_lo + P_lo.Y_hi is
// accumulated in FP32 by three tcgen05.mma kind::f16 per 16-deep K step
// (the dropped P_lo.Y_lo term is ~2^-16 relative).  The residual pass uses
// y = hi + lo.
//
// Per CTA (256 threads, one 64-vertex tile): the tile of Y (hi and lo,
// K-major, no swizzle, 8x16-byte core matrices) stays in shared memory; for
// each group of 16 designs (M = 128 rows) the pseudoinverse rows stream
// through a 32-deep K chunk, thread 0 issues the MMAs, tcgen05.commit
// arrives on an mbarrier (bounded wait), warps 0-3 read the accumulator with
// tcgen05.ld into shared memory and all warps run the epilogue.
#include <cuda_bf16.h>

#include <algorithm>

#include "common.cuh"

namespace tfgb {

constexpr int kTcThreads = 256;
constexpr int kTcN = 64;        // vertices per CTA (MMA N)
constexpr int kTcM = 128;       // design rows per MMA (16 designs x 8)
constexpr int kTcKPad = 8;      // rows per design in the stacked operand
constexpr int kTcKC = 32;       // K elements per A chunk (2 MMA K steps)
constexpr int kTcMaxN = 640;    // subjects supported by the shared-memory tile
constexpr int kBetaLd = kTcN + 1;
constexpr long long kTcWaitLimit = 1LL << 26;

// --- PTX wrappers -----------------------------------------------------------
__device__ inline uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
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

__device__ inline void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ inline void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ inline void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

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

// --- operand preparation --------------------------------------------------
// dst_hi/lo [rows][ld_dst] = split of src [rows][cols] (row stride ld_src),
// zero past cols.  Optional transpose: src is [cols][rows] (Y stored n x V).
__global__ void split_bf16_kernel(const float* __restrict__ src, int64_t ld_src, int transpose, int64_t rows,
                                  int cols, int ld_dst, __nv_bfloat16* __restrict__ hi,
                                  __nv_bfloat16* __restrict__ lo) {
  const int64_t total = rows * ld_dst;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / ld_dst;
    const int c = static_cast<int>(i % ld_dst);
    float x = 0.0f;
    if (c < cols) x = transpose ? src[(int64_t)c * ld_src + r] : src[r * ld_src + c];
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    hi[i] = h;
    lo[i] = __float2bfloat16_rn(x - __bfloat162float(h));
  }
}

// --- the GEMM + epilogue ----------------------------------------------------
struct TcArgs {
  const __nv_bfloat16* y_hi;  // [V][n_pad]
  const __nv_bfloat16* y_lo;
  const __nv_bfloat16* p_hi;  // [G*8][n_pad]
  const __nv_bfloat16* p_lo;
  const float* X;             // [G][n][kmax]
  const float* invdiag;       // [G][kmax]
  const float* dof;           // [G]
  const int32_t* coef;
  float* t_out;               // [G][n_coef][ldt]
  int64_t ldt;
  int64_t V;
  int32_t n, n_pad, G, kmax, n_coef;
  int32_t* err;
};

// Shared memory layout (bytes): [0, A) A chunk hi+lo, then the Y tile hi+lo,
// then beta, then the mbarrier and the TMEM address.  A comes first so that
// every descriptor-addressed read stays inside this CTA's allocation.
__host__ __device__ inline int tc_a_bytes() { return 2 * kTcM * kTcKC * 2; }
__host__ __device__ inline int tc_y_bytes(int n_pad) { return 2 * kTcN * n_pad * 2; }
__host__ __device__ inline int tc_beta_bytes() { return kTcM * kBetaLd * 4; }
__host__ __device__ inline int tc_smem_bytes(int n_pad) {
  return tc_a_bytes() + tc_y_bytes(n_pad) + tc_beta_bytes() + 64;
}

__global__ void __launch_bounds__(kTcThreads, 1) glm_tc_kernel(TcArgs a) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* sA = sm;                                       // hi: [0, A/2), lo: [A/2, A)
  unsigned char* sY = sm + tc_a_bytes();                        // hi then lo
  float* sBeta = reinterpret_cast<float*>(sm + tc_a_bytes() + tc_y_bytes(a.n_pad));
  uint64_t* sBar = reinterpret_cast<uint64_t*>(sm + tc_a_bytes() + tc_y_bytes(a.n_pad) + tc_beta_bytes());
  uint32_t* sTmem = reinterpret_cast<uint32_t*>(sBar + 1);
  const int tid = threadIdx.x, warp = tid / 32;
  const int64_t v0 = (int64_t)blockIdx.x * kTcN;
  const int kb_total = a.n_pad / 8;
  const int a_half = kTcM * kTcKC * 2;
  const int y_half = kTcN * a.n_pad * 2;

  // TMEM: 64 fp32 columns (one N = 64 accumulator), allocated by warp 0
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(smem_addr(sTmem))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(smem_addr(sBar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // Y tile -> core-matrix layout: (kb, nb) at (kb*8 + nb)*128, row v%8 at +16*(v%8)
  for (int i = tid; i < kTcN * kb_total; i += kTcThreads) {
    const int v = i / kb_total, kb = i % kb_total;
    const int off = (kb * 8 + v / 8) * 128 + (v % 8) * 16;
    uint4 h = make_uint4(0, 0, 0, 0), l = make_uint4(0, 0, 0, 0);
    if (v0 + v < a.V) {
      h = *reinterpret_cast<const uint4*>(a.y_hi + (v0 + v) * a.n_pad + kb * 8);
      l = *reinterpret_cast<const uint4*>(a.y_lo + (v0 + v) * a.n_pad + kb * 8);
    }
    *reinterpret_cast<uint4*>(sY + off) = h;
    *reinterpret_cast<uint4*>(sY + y_half + off) = l;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *sTmem;
  const uint32_t bar = smem_addr(sBar);
  const uint32_t idesc = make_idesc(kTcM, kTcN);
  const uint32_t aBase = smem_addr(sA), yBase = smem_addr(sY);
  uint32_t phase = 0;
  const int n_mt = (a.G * kTcKPad + kTcM - 1) / kTcM;

  for (int mt = 0; mt < n_mt; ++mt) {
    for (int kc = 0; kc < a.n_pad / kTcKC; ++kc) {
      // A chunk: rows of this M tile, K [kc*32, kc*32+32): (kb, mb) at (kb*16 + mb)*128
      for (int i = tid; i < kTcM * (kTcKC / 8); i += kTcThreads) {
        const int r = i / (kTcKC / 8), kb = i % (kTcKC / 8);
        const int64_t gr = (int64_t)mt * kTcM + r;
        const int off = (kb * 16 + r / 8) * 128 + (r % 8) * 16;
        uint4 h = make_uint4(0, 0, 0, 0), l = make_uint4(0, 0, 0, 0);
        if (gr < (int64_t)a.G * kTcKPad) {
          h = *reinterpret_cast<const uint4*>(a.p_hi + gr * a.n_pad + kc * kTcKC + kb * 8);
          l = *reinterpret_cast<const uint4*>(a.p_lo + gr * a.n_pad + kc * kTcKC + kb * 8);
        }
        *reinterpret_cast<uint4*>(sA + off) = h;
        *reinterpret_cast<uint4*>(sA + a_half + off) = l;
      }
      fence_proxy_async();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
#pragma unroll
        for (int s = 0; s < kTcKC / 16; ++s) {
          const int q = kc * (kTcKC / 16) + s;  // global 16-deep K step
          const uint64_t ah = make_desc(aBase + s * 2 * 2048, 2048, 128);
          const uint64_t al = make_desc(aBase + a_half + s * 2 * 2048, 2048, 128);
          const uint64_t bh = make_desc(yBase + q * 2 * 1024, 1024, 128);
          const uint64_t bl = make_desc(yBase + y_half + q * 2 * 1024, 1024, 128);
          mma_bf16(tmem, ah, bh, idesc, (kc | s) ? 1u : 0u);
          mma_bf16(tmem, ah, bl, idesc, 1u);
          mma_bf16(tmem, al, bh, idesc, 1u);
        }
        mma_commit(bar);
      }
      // bounded wait for the MMAs of this chunk (they also free the A buffer)
      long long it = 0;
      while (!mbar_try_wait(bar, phase)) {
        if (++it > kTcWaitLimit) {
          if (tid == 0) atomicCAS(a.err, 0, kDevLoopLimit);
          break;
        }
      }
      phase ^= 1u;
      tc_fence_after();
      __syncthreads();
    }
    // accumulator -> shared (warps 0-3 own TMEM lanes 32w..32w+31 = rows)
    if (warp < 4) {
      float buf[16];
#pragma unroll
      for (int c = 0; c < kTcN / 16; ++c) {
        tmem_ld16(tmem + (static_cast<uint32_t>(warp * 32) << 16) + c * 16, buf);
        const int row = warp * 32 + (tid % 32);
#pragma unroll
        for (int j = 0; j < 16; ++j) sBeta[row * kBetaLd + c * 16 + j] = buf[j];
      }
    }
    tc_fence_before();
    __syncthreads();
    // epilogue: 16 designs x 64 vertices, 4 vertices per thread
    {
      const int d = tid / 16;
      const int vb = (tid % 16) * 4;
      const int64_t g = (int64_t)mt * (kTcM / kTcKPad) + d;
      if (g < a.G) {
        const int kmax = a.kmax;
        float beta[kTcKPad][4];
#pragma unroll
        for (int j = 0; j < kTcKPad; ++j)
#pragma unroll
          for (int c = 0; c < 4; ++c) beta[j][c] = (j < kmax) ? sBeta[(d * kTcKPad + j) * kBetaLd + vb + c] : 0.0f;
        float rss[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        const float* xg = a.X + g * a.n * kmax;
        const __nv_bfloat16* yh = reinterpret_cast<const __nv_bfloat16*>(sY);
        const __nv_bfloat16* yl = reinterpret_cast<const __nv_bfloat16*>(sY + y_half);
        for (int s = 0; s < a.n; ++s) {
          float xv[kTcKPad];
#pragma unroll
          for (int j = 0; j < kTcKPad; ++j) xv[j] = (j < kmax) ? __ldg(xg + (int64_t)s * kmax + j) : 0.0f;
          const int kb = s / 8, kk = s % 8;
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int v = vb + c;
            const int e = ((kb * 8 + v / 8) * 128 + (v % 8) * 16) / 2 + kk;
            float r = __bfloat162float(yh[e]) + __bfloat162float(yl[e]);
#pragma unroll
            for (int j = 0; j < kTcKPad; ++j) r = fmaf(-xv[j], beta[j][c], r);
            rss[c] = fmaf(r, r, rss[c]);
          }
        }
        const float inv_dof = 1.0f / a.dof[g];
        for (int ci = 0; ci < a.n_coef; ++ci) {
          const int j = a.coef[ci];
          const float dj = a.invdiag[g * kmax + j];
          float* dst = a.t_out + (g * a.n_coef + ci) * a.ldt + v0 + vb;
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            if (v0 + vb + c < a.V) {
              float bj = 0.0f;
#pragma unroll
              for (int jj = 0; jj < kTcKPad; ++jj)
                if (jj == j) bj = beta[jj][c];
              dst[c] = bj / sqrtf(rss[c] * inv_dof * dj);
            }
          }
        }
      }
    }
    __syncthreads();
    tc_fence_after();
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem) : "memory");
  }
}

}  // namespace tfgb

extern "C" {

int glm_split_bf16(const float* src, int64_t ld_src, int32_t transpose, int64_t rows, int32_t cols,
                   int32_t ld_dst, void* hi, void* lo, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(src && hi && lo, "NULL pointer");
  TFGB_CHECK_ARG(rows >= 0 && cols >= 0 && ld_dst >= cols && ld_dst % 8 == 0, "bad sizes");
  if (rows == 0) return TFCE_OK;
  const int64_t total = rows * ld_dst;
  const unsigned blocks = static_cast<unsigned>(std::min<int64_t>((total + 255) / 256, 152 * 32));
  tfgb::split_bf16_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      src, ld_src, transpose, rows, cols, ld_dst, static_cast<__nv_bfloat16*>(hi),
      static_cast<__nv_bfloat16*>(lo));
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

int glm_tstat_tc(const void* y_hi, const void* y_lo, int32_t n, int32_t n_pad, int64_t V, const void* p_hi,
                 const void* p_lo, const float* X, const float* invdiag, const float* dof, int32_t G,
                 int32_t kmax, const int32_t* coef, int32_t n_coef, float* t_out, int64_t ldt, int32_t* err,
                 void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(y_hi && y_lo && p_hi && p_lo && X && invdiag && dof && coef && t_out && err, "NULL pointer");
  TFGB_CHECK_ARG(n > 0 && n_pad >= n && n_pad % tfgb::kTcKC == 0, "n_pad must be >= n and a multiple of 32");
  TFGB_CHECK_ARG(n_pad <= tfgb::kTcMaxN, "more than 640 subjects: use glm_tstat");
  TFGB_CHECK_ARG(kmax >= 1 && kmax <= tfgb::kTcKPad, "kmax must be in [1, 8]");
  TFGB_CHECK_ARG(n_coef >= 1 && V >= 0 && G >= 0 && ldt >= V, "bad sizes");
  if (V == 0 || G == 0) return TFCE_OK;
  const int smem = tfgb::tc_smem_bytes(n_pad);
  TFGB_CUDA(cudaFuncSetAttribute(tfgb::glm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  tfgb::TcArgs a{};
  a.y_hi = static_cast<const __nv_bfloat16*>(y_hi);
  a.y_lo = static_cast<const __nv_bfloat16*>(y_lo);
  a.p_hi = static_cast<const __nv_bfloat16*>(p_hi);
  a.p_lo = static_cast<const __nv_bfloat16*>(p_lo);
  a.X = X;
  a.invdiag = invdiag;
  a.dof = dof;
  a.coef = coef;
  a.t_out = t_out;
  a.ldt = ldt;
  a.V = V;
  a.n = n;
  a.n_pad = n_pad;
  a.G = G;
  a.kmax = kmax;
  a.n_coef = n_coef;
  a.err = err;
  const unsigned grid = static_cast<unsigned>((V + tfgb::kTcN - 1) / tfgb::kTcN);
  tfgb::glm_tc_kernel<<<grid, tfgb::kTcThreads, smem, static_cast<cudaStream_t>(stream)>>>(a);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

}  // extern "C"
