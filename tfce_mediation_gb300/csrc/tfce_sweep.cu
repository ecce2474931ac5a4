// TFCE sweep over adjacency sets, batched: the GB300 replacement of
// tfce_mediation/lib/fast_tfce.hpp:11-95 (reached through
// tfce_mediation/tfce.pyx:44-45) and of the per-permutation scaling/max of
// tfce_mediation/pyfunc.py:107-126.
//
// One work item = (map, sign, segment).  One CTA sweeps one item at a time and
// pulls the next from a global queue (persistent grid sized to the resident
// CTA count).  Per item:
//   1. maxT = segment max; the threshold table T_i (float recurrence
//      T -= maxT/100 while T >= 0, fast_tfce.hpp:34-39) and HH_i = T_i^H are
//      built in shared memory;
//   2. every vertex gets the step at which it activates (first i with
//      x > T_i, strict as fast_tfce.hpp:41) and vertices are bucketed by that
//      step (counting sort, no full sort: order inside a step does not change
//      the partition);
//   3. per step: (U) new vertices are unioned with active neighbours by a
//      lock-free union-find in the bucket-position space (CAS links the
//      larger root under the smaller, so parent[x] < x and walks end).  A
//      thread takes the next new vertex from a shared cursor, walks the roots
//      of all its effective neighbours in lockstep (one round of loads per
//      hop; path halving in the exact mode) and links every distinct root
//      under the smallest with CASes issued together; a lost race falls back
//      to a general unite; (S) the roots that were linked this step hand their
//      extent to their final root and point at it; (A) every active vertex
//      adds (float)(extent^E * HH_i) to its own
//      accumulator, in threshold order -- the reference's per-vertex
//      arithmetic, so results are bit-identical to it;
//   4. the map is scaled by max/100 (and vdensity), reduced to its max, and
//      optionally written out.
// Every walk and retry loop is bounded; a bound sets an error word and the
// kernel runs on to its exit.
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace tfgb {

#ifdef TFGB_PHASE_PROFILE
// Debug-only: clock64 cycles spent per phase, summed over items (thread 0).
__device__ unsigned long long g_phase_cycles[8];
#define TFGB_PHASE_MARK(k)                                              \
  do {                                                                  \
    if (threadIdx.x == 0) {                                             \
      const long long _now = clock64();                                 \
      atomicAdd(&g_phase_cycles[k], (unsigned long long)(_now - _pt));  \
      _pt = _now;                                                       \
    }                                                                   \
  } while (0)
// Debug-only event counters: [0] unite calls, [1] CAS attempts, [2] CAS
// failures, [3] find hops, [4] halving writes, [5] list entries checked.
__device__ unsigned long long g_dbg_counts[8];
// Debug-only: cycles of each step's (U+S+A) by threshold index.
__device__ unsigned long long g_step_cycles[128];
#define TFGB_COUNT(k, n) atomicAdd(&g_dbg_counts[k], (unsigned long long)(n))
#else
#define TFGB_PHASE_MARK(k) do { } while (0)
#define TFGB_COUNT(k, n) do { } while (0)
#endif

constexpr int kMaxSteps = 128;
#ifndef TFGB_SWEEP_THREADS
#define TFGB_SWEEP_THREADS 512
#endif
#ifndef TFGB_ACTIVE_BITMAP
#define TFGB_ACTIVE_BITMAP 1
#endif
// largest activity bitmap kept in shared memory (segments up to 393,216 vertices)
constexpr int kBitmapMaxBytes = 48 * 1024;
#ifndef TFGB_SWEEP_MINBLOCKS
#define TFGB_SWEEP_MINBLOCKS 3  // 3 x 512 threads per SM (40 registers; a few spills)
#endif
#ifndef TFGB_UBATCH
#define TFGB_UBATCH 6
#endif
#ifndef TFGB_ALANES
#define TFGB_ALANES 1
#endif
// path halving in the maxima-only form (no potential chains to preserve)
#ifndef TFGB_MAX_HALVE
#define TFGB_MAX_HALVE 0
#endif
#ifndef TFGB_MAX_REC8  // maxima-only form: 8-byte {float sum, extent} records
#define TFGB_MAX_REC8 1
#endif
constexpr int kSweepThreads = TFGB_SWEEP_THREADS;
constexpr int kUBatch = TFGB_UBATCH;   // list entries of one vertex looked up together
constexpr int kALanes = TFGB_ALANES;   // positions per thread per accumulation round
#ifndef TFGB_SLANES
#define TFGB_SLANES 1
#endif
constexpr int kSLanes = TFGB_SLANES;   // dead roots per thread per size round
constexpr uint32_t kOneWay = 0x80000000u;   // entry whose reverse entry is missing
constexpr uint32_t kIndexMask = 0x7fffffffu;
constexpr uint32_t kInactiveKey = 0xffffffffu;
constexpr int kPosBits = 24;                 // key = step << 24 | position
constexpr int32_t kMaxSegVertices = (1 << kPosBits) - 1;
constexpr int kWalkLimit = 1 << 26;

struct SweepArgs {
  const int64_t* offsets;
  const uint32_t* indices;
  const float* stats;
  int64_t map_stride;
  int32_t n_maps;
  int32_t n_signs;
  int32_t n_seg;
  const int64_t* seg_off;
  const float* seg_H;
  const float* seg_E;
  const float* vdensity;
  int32_t floor_zero;
  float* out_max;
  float* out_maps;
  int32_t out_mode;
  int32_t* labels;
  int32_t* extents;
  int32_t* n_steps_out;
  int32_t label_cap;
  char* ws;
  int64_t ws_slot_bytes;
  int32_t vcap;
  int32_t* counter;
  int32_t* err;
  int32_t n_items;
  const int32_t* item_order;
  // Checked variant only (caller-provided device CSR): vertex and entry counts
  // the kernel validates segment ranges and list extents against.
  int32_t n_vertices;
  int64_t n_entries;
  // words of the shared-memory activity bitmap (dynamic shared memory), 0 = none
  int32_t bm_words;
  // Threshold groups (nullable): segments with the same thr_group[seg] share
  // one threshold table, built from the largest of their maxima -- the sweep
  // of one merged adjacency over several surfaces (tm_func.py:68-78), whose
  // dT is the merged image's max / 100.  seg_max [n_maps][n_signs][n_seg]
  // holds every segment's maximum (segment_max_kernel); the scale stays each
  // segment's own max / 100 (tm_func.py:84-91).
  const int32_t* thr_group;
  const float* seg_max;
  // segments by decreasing size (nullable): the order items are handed out in
  const int32_t* seg_rank;
};

// Per-component mode: the increments so far (root) or the potential to the
// root joined (dead root) and the extent of a position, in one 16-byte record
// so that the size and accumulation phases touch one sector per position.
struct alignas(16) Rec {
  double w;
  int32_t size;
  int32_t pad;
};

// Maxima-only form: {sum, extent} of a position in 8 bytes (in the Rec region
// of the slot; four records per sector).  The sum is a float: rounding is
// monotone, so fl(max(a, b) + x) = max(fl(a + x), fl(b + x)), and the largest
// float sum kept per component equals the largest per-vertex float
// accumulation of its members (fast_tfce.hpp:77-82) bit for bit.
struct alignas(8) Rec8 {
  float w;  // >= 0: ordered as its bit pattern
  int32_t size;
};

struct Slot {
  uint32_t* key;
  int32_t* order;
  int32_t* parent;
  int32_t* size;
  float* acc;
  int32_t* dead;
  // per-component accumulation only
  int32_t* roots_a;  // live roots after the previous threshold ...
  int32_t* roots_b;  // ... and after this one (swapped every step)
  Rec* rec;          // {W, extent} per position
};

__host__ __device__ inline int64_t align_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

__host__ __device__ inline int64_t slot_bytes(int32_t vcap) {
  return 6 * align_up((int64_t)vcap * 4, 256);
}

// Per-component accumulation adds two root lists and a 16-byte {W, extent}
// record per vertex to the six int32/float arrays of the exact mode.
__host__ __device__ inline int64_t slot_bytes_lazy(int32_t vcap) {
  return 8 * align_up((int64_t)vcap * 4, 256) + align_up((int64_t)vcap * 16, 256);
}

__device__ inline Slot make_slot(char* base, int32_t vcap) {
  const int64_t s = align_up((int64_t)vcap * 4, 256);
  Slot sl;
  sl.roots_a = reinterpret_cast<int32_t*>(base + 6 * s);
  sl.roots_b = reinterpret_cast<int32_t*>(base + 7 * s);
  sl.rec = reinterpret_cast<Rec*>(base + 8 * s);
  sl.key = reinterpret_cast<uint32_t*>(base);
  sl.order = reinterpret_cast<int32_t*>(base + s);
  sl.parent = reinterpret_cast<int32_t*>(base + 2 * s);
  sl.size = reinterpret_cast<int32_t*>(base + 3 * s);
  sl.acc = reinterpret_cast<float*>(base + 4 * s);
  sl.dead = reinterpret_cast<int32_t*>(base + 5 * s);
  return sl;
}

__device__ inline void set_err(int32_t* err, int32_t code) { atomicCAS(err, 0, code); }

// dynamic shared memory of the activity bitmap for segments of up to vmax
// vertices (0 when it would not fit: the union phase then loads every key)
inline int bitmap_bytes(int64_t vmax) {
  const int64_t b = (vmax + 31) / 32 * 4;
  return (TFGB_ACTIVE_BITMAP && b <= kBitmapMaxBytes) ? static_cast<int>(b) : 0;
}

// Union-find state of an item is private to the one CTA (one SM) sweeping it,
// so loads and stores of it are relaxed at CTA scope: coherent with the
// CTA's own CAS/atomics under the PTX memory model, and free to be served
// from L1 (the hot roots of large components are read by every thread).
#ifndef TFGB_STATE_GLOBAL_SCOPE
__device__ inline int32_t ld_state(const int32_t* p) {
  int32_t v;
  asm volatile("ld.relaxed.cta.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ inline void st_state(int32_t* p, int32_t v) {
  asm volatile("st.relaxed.cta.global.s32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}
#else
__device__ inline int32_t ld_state(const int32_t* p) { return __ldcg(p); }
__device__ inline void st_state(int32_t* p, int32_t v) { __stcg(p, v); }
#endif

// Root of x, halving the path on the way: every non-root visited is
// re-pointed to its grandparent.  Only roots are ever linked (by CAS), and a
// non-root's new parent is one of its ancestors, so concurrent walks and links
// stay consistent.  parent[] entries only point to smaller positions, so the
// walk ends; the limit is a second guard.
template <bool kHalve = true>
__device__ inline int32_t find_root(int32_t* parent, int32_t x, int32_t* err) {
  for (int it = 0; it < kWalkLimit; ++it) {
    const int32_t p = ld_state(parent + x);
    TFGB_COUNT(3, 1);
    if (p == x) return x;
    const int32_t g = ld_state(parent + p);
    TFGB_COUNT(3, 1);
    if (g == p) return p;
    if (kHalve) st_state(parent + x, g);
    TFGB_COUNT(4, 1);
    x = g;
  }
  set_err(err, kDevLoopLimit);
  return x;
}

// Join the component of root-hint `a` with position b; returns the root of
// the joined component (a hint: another thread may link it later).  A linked
// root older than fresh_lo is appended to the dead list.
template <bool kHalve = true>
__device__ inline int32_t unite(int32_t* parent, int32_t a, int32_t b, int32_t* dead,
                                int32_t* n_dead, int32_t fresh_lo, int32_t* err) {
  TFGB_COUNT(0, 1);
  for (int it = 0; it < kWalkLimit; ++it) {
    a = find_root<kHalve>(parent, a, err);
    b = find_root<kHalve>(parent, b, err);
    if (a == b) return a;
    const int32_t hi = max(a, b), lo = min(a, b);
    TFGB_COUNT(1, 1);
    const int32_t old = atomicCAS(parent + hi, hi, lo);
    if (old != hi) TFGB_COUNT(2, 1);
    if (old == hi) {
      // roots activated at this step (positions >= fresh_lo) are found by the
      // size phase in the step's own position range; older ones are listed
      if (hi < fresh_lo) dead[atomicAdd(n_dead, 1)] = hi;
      return lo;
    }
  }
  set_err(err, kDevLoopLimit);
  return a;
}

// (float)(extent^E * HH) with the reference's types: pow in double, product in
// double, one rounding to float (fast_tfce.hpp:77).  For E == 1 the double
// product of an integer < 2^24 and a float is exact, so one float multiply
// rounds identically.
__device__ inline float increment(int32_t extent, float E, int e_mode, float HH) {
  if (e_mode == 1) return __fmul_rn(static_cast<float>(extent), HH);
  double pe;
  if (e_mode == 2) pe = sqrt(static_cast<double>(extent));
  else if (e_mode == 3) pe = static_cast<double>(extent) * static_cast<double>(extent);
  else pe = pow(static_cast<double>(extent), static_cast<double>(E));
  return __double2float_rn(__dmul_rn(pe, static_cast<double>(HH)));
}

// HH = pow(T, H) as a float (fast_tfce.hpp:70), correctly rounded: T*T for
// H == 2 (exact product, one rounding), otherwise the double-precision power
// rounded once to float.  The reference calls the host libm's powf, which is
// not always correctly rounded (glibc: <= 0.82 ulp), so at rare thresholds
// its HH can sit one float ulp away from this value.
__device__ inline float pow_h(float T, float H) {
  if (H == 2.0f) return __fmul_rn(T, T);
  if (H == 1.0f) return T;
  return __double2float_rn(pow(static_cast<double>(T), static_cast<double>(H)));
}

__device__ inline float block_max(float v, float* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (l < (int)(blockDim.x >> 5)) ? red[l] : -INFINITY;
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (l == 0) red[0] = v;
  }
  __syncthreads();
  const float r = red[0];
  __syncthreads();
  return r;
}

// kChecked = false: the handle's cleaned CSR (validated on the host, entries
// whose reverse is missing flagged).  kChecked = true: a CSR the caller keeps
// on the device, unvalidated and unflagged -- segment ranges and list extents
// are checked here, and the insertion-order rule is applied to every
// same-step entry (for a symmetric pair exactly one direction passes it, so
// the partition is the same).
//
// kLazy = false: the reference's arithmetic -- every active vertex adds its
// float increment to its own float accumulator at every threshold, so results
// are bit-identical to the reference sweep.  kLazy = true: per-component
// accumulation -- each live root adds its component's increment to a double
// once per threshold; a root that is linked keeps its potential relative to
// the root it joins, and a vertex's value is the sum of potentials along its
// parent chain (no path halving in this mode, so a dead root's parent stays
// the root it joined), rounded to float once.  Per threshold that is O(live
// components) instead of O(active vertices); the result is the exact sum of
// the same float increments, so it differs from the reference only by the
// reference's own float summation error.
//
// kMaxOnly (with kLazy): only the scaled maxima are wanted and no vertex
// weights apply.  Every vertex of a component gets the same increment from
// the threshold it joins it on, so the largest TFCE in a component is the
// largest sum accumulated by any of the components merged into it, plus the
// merged component's own increments since: a root keeps that largest sum
// (a linked root hands its sum to its final root by atomic max) and the
// map's maximum is the largest sum among the last live roots.  No potentials
// are kept, so there is no per-vertex resolve pass.
//
// kMinBlocks: resident CTAs per SM the register budget is cut for (3: 40
// registers with a few spills, the most items in flight; 2: 64 registers, no
// spills) -- the sweep's CTA shape, chosen per study by the autotuner.
template <bool kChecked, bool kLazy, bool kMaxOnly = false, int kMinBlocks = TFGB_SWEEP_MINBLOCKS>
__global__ void __launch_bounds__(kSweepThreads, kMinBlocks) tfce_sweep_kernel(SweepArgs a) {
  static_assert(!kMaxOnly || kLazy, "the maxima-only form is a per-component form");
  __shared__ float sT[kMaxSteps];
  __shared__ float sHH[kMaxSteps];
  __shared__ int32_t sCnt[kMaxSteps + 1];
  __shared__ int32_t sStart[kMaxSteps + 1];
  __shared__ float sRed[32];
  __shared__ int32_t sItem, sL, sNDead, sNRoots, sNext, sGrab, sGrabS, sGrabA;
  // bit v set once vertex v is active (its activation step <= the current
  // step): the union phase loads a neighbour's key only when it is set
  extern __shared__ uint32_t sAct[];
  const bool use_bm = TFGB_ACTIVE_BITMAP && a.bm_words > 0;

  Slot sl = make_slot(a.ws + (int64_t)blockIdx.x * a.ws_slot_bytes, a.vcap);
  const int tid = threadIdx.x, nth = blockDim.x;
  // Per-component mode keeps every dead root's parent at the root it joined
  // (no path halving), so parent[] is also the chain of the potentials; the
  // exact mode halves paths.
  constexpr bool kHalve = !kLazy || (kMaxOnly && TFGB_MAX_HALVE);
  // Maxima-only form: float sums and extents in 8-byte records
  constexpr bool kR8 = kMaxOnly && TFGB_MAX_REC8;
  Rec8* const rec8 = reinterpret_cast<Rec8*>(sl.rec);
  // and {vertex, packed list} of a position in one 8-byte record (the second
  // half of the Rec region), so that bucketing scatters one store per vertex
  int2* const vtx8 = reinterpret_cast<int2*>(sl.rec) + a.vcap;
#ifdef TFGB_PHASE_PROFILE
  long long _pt = clock64();
#endif

  for (;;) {
    if (tid == 0) sItem = atomicAdd(a.counter, 1);
    __syncthreads();
    const int32_t qi = sItem;
    __syncthreads();
    if (qi >= a.n_items) break;
    int32_t item = a.item_order ? a.item_order[qi] : qi;
    if (a.seg_rank) {  // largest segments first; n_items is a multiple of n_seg
      const int32_t per_seg = a.n_items / a.n_seg;
      item = (qi % per_seg) * a.n_seg + a.seg_rank[qi / per_seg];
    }
    const int32_t seg = item % a.n_seg;
    const int32_t ms = item / a.n_seg;  // map * n_signs + sign
    const int32_t sgn = ms % a.n_signs;
    const int32_t map = ms / a.n_signs;
    const float sign = sgn ? -1.0f : 1.0f;
    const int64_t v0 = a.seg_off[seg];
    const int32_t Vs = static_cast<int32_t>(a.seg_off[seg + 1] - v0);
    if constexpr (kChecked) {
      const int64_t len = a.seg_off[seg + 1] - v0;
      if (v0 < 0 || len < 0 || len > a.vcap || v0 + len > a.n_vertices) {
        if (tid == 0) {
          set_err(a.err, kDevBadIndex);
          if (a.out_max) a.out_max[item] = 0.0f;
        }
        continue;
      }
    }
    const float H = a.seg_H[seg], E = a.seg_E[seg];
    const int e_mode = (E == 1.0f) ? 1 : (E == 0.5f) ? 2 : (E == 2.0f) ? 3 : 0;
    const float* x = a.stats + (int64_t)map * a.map_stride + v0;
    const int64_t seg_e0 = a.offsets[v0];
    const float* vd = a.vdensity ? a.vdensity + v0 : nullptr;
    float* omap = a.out_maps ? a.out_maps + (int64_t)ms * (a.seg_off[a.n_seg]) + v0 : nullptr;

    // ---- 1. maximum and threshold table
    float mx = -INFINITY;
    for (int32_t v = tid; v < Vs; v += nth) {
      const float xv = sign * x[v];
      if (isfinite(xv)) mx = fmaxf(mx, xv);
    }
    mx = block_max(mx, sRed);
    if (a.floor_zero) mx = fmaxf(mx, 0.0f);
    if (tid == 0) {
      // the threshold table's maximum: this segment's, or its group's
      float tmx = mx;
      if (a.thr_group) {
        const int32_t g = a.thr_group[seg];
        const float* gm = a.seg_max + (int64_t)ms * a.n_seg;
        tmx = -INFINITY;
        for (int32_t s2 = 0; s2 < a.n_seg; ++s2)
          if (a.thr_group[s2] == g) tmx = fmaxf(tmx, gm[s2]);
      }
      int L = 0;
      if (tmx > 0.0f && isfinite(tmx)) {
        const float dT = __fdiv_rn(tmx, 100.0f);
        float T = tmx;
        while (T >= 0.0f) {
          if (L >= kMaxSteps) {
            set_err(a.err, kDevTooManySteps);
            L = 0;
            break;
          }
          sT[L] = T;
          sHH[L] = pow_h(T, H);
          ++L;
          T = __fsub_rn(T, dT);
        }
      }
      sL = L;
      if (a.n_steps_out) *a.n_steps_out = L;
    }
    for (int i = tid; i <= kMaxSteps; i += nth) sCnt[i] = 0;
    if (use_bm)
      for (int32_t w = tid; w < (Vs + 31) / 32; w += nth) sAct[w] = 0u;
    __syncthreads();
    TFGB_PHASE_MARK(0);
    const int L = sL;
    const float scale = isfinite(mx) ? __fdiv_rn(mx, 100.0f) : 0.0f;

    // ---- 2. activation step per vertex, bucket histogram
    for (int32_t v = tid; v < Vs; v += nth) {
      const float xv = sign * x[v];
      int lv = L;  // L == never active
      if (L > 0 && xv > sT[L - 1]) {
        int lo = 0, hi = L - 1;  // smallest i with xv > T[i]; T decreasing
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (xv > sT[mid]) hi = mid;
          else lo = mid + 1;
        }
        lv = lo;
      }
      sl.key[v] = static_cast<uint32_t>(lv);  // provisional: step only
      if (lv < L) {
        const unsigned mask = __activemask();
        const unsigned peers = __match_any_sync(mask, lv);
        const int leader = __ffs(peers) - 1;
        if ((tid & 31) == leader) atomicAdd(&sCnt[lv], __popc(peers));
      }
    }
    __syncthreads();
    if (tid == 0) {
      int32_t s = 0;
      for (int i = 0; i < L; ++i) {
        sStart[i] = s;
        s += sCnt[i];
        sCnt[i] = 0;  // reused as fill cursor
      }
      sStart[L] = s;
      sNDead = 0;
      sNRoots = 0;
      sNext = 0;
      sGrab = 0;
      sGrabS = 0;
    }
    __syncthreads();
    const int32_t n_act = sStart[L];
    for (int32_t v = tid; v < Vs; v += nth) {
      const int lv = static_cast<int>(sl.key[v]);
      uint32_t key = kInactiveKey;
      if (lv < L) {
        const unsigned mask = __activemask();
        const unsigned peers = __match_any_sync(mask, lv);
        const int leader = __ffs(peers) - 1;
        const int lane = tid & 31;
        int base = 0;
        if (lane == leader) base = atomicAdd(&sCnt[lv], __popc(peers));
        base = __shfl_sync(peers, base, leader);
        const int32_t p = sStart[lv] + base + __popc(peers & ((1u << lane) - 1u));
        key = (static_cast<uint32_t>(lv) << kPosBits) | static_cast<uint32_t>(p);
        if (use_bm && lv == 0) atomicOr(&sAct[v >> 5], 1u << (v & 31));
        if constexpr (!kR8) sl.order[p] = v;
        // maxima-only form: parents and records are set one step ahead, for
        // a step's contiguous positions at once (below and in (A'))
        if constexpr (!kR8) sl.parent[p] = p;
        if constexpr (kLazy) {
          if constexpr (!kR8) sl.rec[p] = Rec{0.0, 1, 0};
          // the vertex's list (start relative to the segment's, degree) by
          // position, so the union phase reads it without a dependent load;
          // -1: out of the packed range, read the offsets
          const int64_t e0 = a.offsets[v0 + v], deg = a.offsets[v0 + v + 1] - e0, rel = e0 - seg_e0;
          const int32_t packed =
              (deg <= 63 && rel >= 0 && rel < (int64_t(1) << 25)) ? static_cast<int32_t>((rel << 6) | deg) : -1;
          if constexpr (kR8) vtx8[p] = make_int2(v, packed);
          else reinterpret_cast<int32_t*>(sl.acc)[p] = packed;
        } else {
          sl.size[p] = 1;
          sl.acc[p] = (a.out_mode == 2 && omap) ? omap[v] : 0.0f;
        }
      }
      sl.key[v] = key;
    }
    if constexpr (kR8) {
      if (L > 0)  // the first step's positions (sStart was set before the last barrier)
        for (int32_t q = sStart[0] + tid; q < sStart[1]; q += nth) {
          sl.parent[q] = q;
          rec8[q] = Rec8{0.0f, 1};
        }
    }
    __syncthreads();
    TFGB_PHASE_MARK(1);

    // ---- 3. threshold steps
    int32_t* cur_roots = sl.roots_a;
    int32_t* nxt_roots = sl.roots_b;
    for (int i = 0; i < L; ++i) {
#ifdef TFGB_PHASE_PROFILE
      const long long _ps = clock64();
#define TFGB_STEP_DONE() do { if (threadIdx.x == 0) atomicAdd(&g_step_cycles[i], (unsigned long long)(clock64() - _ps)); } while (0)
#else
#define TFGB_STEP_DONE() do { } while (0)
#endif
      const int32_t s0 = sStart[i], s1 = sStart[i + 1];
      // (U) union newly active vertices with already-active neighbours.  A
      // vertex's list is read kUBatch entries at a time with all their key
      // lookups issued together; the root of the vertex's component is kept
      // as a hint between unions.
      // Batched union: the roots of all effective neighbours of a vertex
      // (positions in cur, -1 = none) and of the vertex's own component
      // (hint rp) are walked in lockstep, one round of loads per hop, then
      // every distinct root other than the smallest is linked under it.  A
      // link is a CAS that succeeds only on a root; a lost race falls back to
      // the general unite.  Returns the root of the joined component (a hint).
      auto walk_link = [&](int32_t (&cur)[kUBatch], int32_t rp) -> int32_t {
        int32_t rr = rp;
        for (int it = 0;; ++it) {
          if (it >= kWalkLimit) {
            set_err(a.err, kDevLoopLimit);
            break;
          }
          int32_t par[kUBatch];
#pragma unroll
          for (int k = 0; k < kUBatch; ++k) par[k] = (cur[k] >= 0) ? ld_state(sl.parent + cur[k]) : cur[k];
          const int32_t pr = ld_state(sl.parent + rr);
          bool walking = (pr != rr);
#pragma unroll
          for (int k = 0; k < kUBatch; ++k) walking |= (par[k] != cur[k]);
          if (!walking) break;
          int32_t gp[kUBatch];
#pragma unroll
          for (int k = 0; k < kUBatch; ++k) gp[k] = (par[k] != cur[k]) ? ld_state(sl.parent + par[k]) : par[k];
          const int32_t gr = (pr != rr) ? ld_state(sl.parent + pr) : pr;
#pragma unroll
          for (int k = 0; k < kUBatch; ++k) {
            if (par[k] != cur[k]) {
              if (kHalve && gp[k] != par[k]) st_state(sl.parent + cur[k], gp[k]);  // halve the path
              cur[k] = gp[k];
            }
          }
          if (pr != rr) {
            if (kHalve && gr != pr) st_state(sl.parent + rr, gr);
            rr = gr;
          }
        }
        int32_t tgt = rr;
#pragma unroll
        for (int k = 0; k < kUBatch; ++k)
          if (cur[k] >= 0) tgt = min(tgt, cur[k]);
        // distinct roots other than the target, each linked once; the
        // CASes are issued together, their results read afterwards
        int32_t lk[kUBatch + 1], old[kUBatch + 1];
        lk[0] = (rr != tgt) ? rr : -1;
#pragma unroll
        for (int k = 0; k < kUBatch; ++k) {
          bool keep = cur[k] >= 0 && cur[k] != tgt && cur[k] != rr;
#pragma unroll
          for (int j = 0; j < k; ++j) keep &= (cur[j] != cur[k]);
          lk[k + 1] = keep ? cur[k] : -1;
        }
#pragma unroll
        for (int m = 0; m <= kUBatch; ++m) old[m] = (lk[m] >= 0) ? atomicCAS(sl.parent + lk[m], lk[m], tgt) : -1;
#pragma unroll
        for (int m = 0; m <= kUBatch; ++m) {
          if (lk[m] < 0) continue;
          if (old[m] == lk[m]) {
            if (lk[m] < s0) sl.dead[atomicAdd(&sNDead, 1)] = lk[m];  // new roots: found by (S) in [s0, s1)
          } else {
            tgt = unite<kHalve>(sl.parent, tgt, lk[m], sl.dead, &sNDead, s0, a.err);
          }
        }
        return tgt;
      };
      // each thread takes the next unprocessed vertex of the step from a
      // shared cursor, so threads with short walks do not wait for slow ones
      for (int32_t p = atomicAdd(&sGrab, 1); p < s1; p = atomicAdd(&sGrab, 1)) {
        int32_t v = -1;  // the vertex: read when needed
        int64_t e0, e1;
        int32_t pk = -1;
        if constexpr (kR8) {
          const int2 r = vtx8[p];
          v = r.x;
          pk = r.y;
        } else if constexpr (kLazy) {
          pk = reinterpret_cast<const int32_t*>(sl.acc)[p];
        }
        if (pk >= 0) {
          e0 = seg_e0 + (pk >> 6);
          e1 = e0 + (pk & 63);
        } else {
          if (v < 0) v = sl.order[p];
          e0 = a.offsets[v0 + v];
          e1 = a.offsets[v0 + v + 1];
        }
        if constexpr (kChecked) {
          if (e0 < 0 || e1 > a.n_entries || e1 < e0) {
            set_err(a.err, kDevBadIndex);
            e0 = e1 = 0;
          }
        }
        int32_t rp = p;
        for (int64_t eb = e0; eb < e1; eb += kUBatch) {
          uint32_t raw[kUBatch], ka[kUBatch];
          int32_t an[kUBatch];
#pragma unroll
          for (int k = 0; k < kUBatch; ++k) raw[k] = (eb + k < e1) ? a.indices[eb + k] : kIndexMask;
          TFGB_COUNT(5, (e1 - eb < kUBatch) ? (e1 - eb) : kUBatch);
#pragma unroll
          for (int k = 0; k < kUBatch; ++k) {
            const int64_t ag = static_cast<int64_t>(raw[k] & kIndexMask) - v0;
            an[k] = static_cast<int32_t>(ag);
            ka[k] = kInactiveKey;
            if (eb + k < e1) {
              // a caller's negative int32 entry has bit 31 set: rejected, not masked
              if (ag < 0 || ag >= Vs || (kChecked && (raw[k] & kOneWay))) set_err(a.err, kDevBadIndex);
              else if (!use_bm || ((sAct[an[k] >> 5] >> (an[k] & 31)) & 1u)) ka[k] = sl.key[an[k]];
            }
          }
          // Batched union: the roots of all effective neighbours in this
          // batch (and of the vertex's own component) are walked in lockstep,
          // one round of loads per hop, then every distinct root other than
          // the smallest is linked under it.  A link is a CAS that succeeds
          // only on a root; a lost race falls back to the general unite.
          int32_t cur[kUBatch];
#pragma unroll
          for (int k = 0; k < kUBatch; ++k) {
            cur[k] = -1;
            if (ka[k] == kInactiveKey) continue;
            const int la = static_cast<int>(ka[k] >> kPosBits);
            if (la > i) continue;
            if (la == i && (kChecked || (raw[k] & kOneWay))) {
              // one-directional entry: effective only if the neighbour was
              // inserted first (larger value; ties by smaller index)
              if (v < 0) v = sl.order[p];  // (set above in the maxima-only form)
              const float xa = sign * x[an[k]], xv = sign * x[v];
              if (!(xa > xv || (xa == xv && an[k] < v))) continue;
            }
            cur[k] = static_cast<int32_t>(ka[k] & ((1u << kPosBits) - 1u));
          }
          bool any = false;
#pragma unroll
          for (int k = 0; k < kUBatch; ++k) any |= (cur[k] >= 0);
          if (!any) continue;
          rp = walk_link(cur, rp);
        }
      }
      __syncthreads();
      if (tid == 0) sGrab = s1;  // the next step's first position
      if (use_bm && i + 1 < L) {
        // the next step's vertices become active (read after two more barriers)
        const int32_t s2 = sStart[i + 2];
        for (int32_t q = s1 + tid; q < s2; q += nth) {
          const int32_t vq = kR8 ? vtx8[q].x : sl.order[q];
          atomicOr(&sAct[vq >> 5], 1u << (vq & 31));
        }
      }
      TFGB_PHASE_MARK(2);
      // (S) linked roots hand their extent to their final root: the listed
      // older roots and the positions of this step that are no longer roots.
      // Each thread takes kSLanes of them per round and walks them in
      // lockstep from their parents; parent[d] is rewritten only when the
      // final root is not already its parent.
      const int32_t nd = sNDead;
      const int32_t nsp = nd + (s1 - s0);
      for (int32_t q0 = atomicAdd(&sGrabS, kSLanes); q0 < nsp; q0 = atomicAdd(&sGrabS, kSLanes)) {
        int32_t d[kSLanes], c[kSLanes], pd[kSLanes];
#pragma unroll
        for (int k = 0; k < kSLanes; ++k) {
          const int32_t q = q0 + k;
          d[k] = (q < nd) ? sl.dead[q] : (q < nsp ? s0 + (q - nd) : -1);
        }
#pragma unroll
        for (int k = 0; k < kSLanes; ++k) {
          pd[k] = (d[k] >= 0) ? ld_state(sl.parent + d[k]) : -1;
          if (pd[k] == d[k]) d[k] = -1;  // still a root
          c[k] = (d[k] >= 0) ? pd[k] : -1;
        }
        for (int it = 0;; ++it) {
          if (it >= kWalkLimit) {
            set_err(a.err, kDevLoopLimit);
            break;
          }
          int32_t par[kSLanes];
#pragma unroll
          for (int k = 0; k < kSLanes; ++k) par[k] = (c[k] >= 0) ? ld_state(sl.parent + c[k]) : c[k];
          bool walking = false;
#pragma unroll
          for (int k = 0; k < kSLanes; ++k) walking |= (par[k] != c[k]);
          if (!walking) break;
          int32_t gp[kSLanes];
#pragma unroll
          for (int k = 0; k < kSLanes; ++k) gp[k] = (par[k] != c[k]) ? ld_state(sl.parent + par[k]) : par[k];
#pragma unroll
          for (int k = 0; k < kSLanes; ++k) {
            if (par[k] != c[k]) {
              if (kHalve && gp[k] != par[k]) st_state(sl.parent + c[k], gp[k]);  // halve the path
              c[k] = gp[k];
            }
          }
        }
        if constexpr (kR8) {
#pragma unroll
          for (int k = 0; k < kSLanes; ++k) {
            if (d[k] < 0) continue;
            // d is no longer a root: no other thread writes its record in this
            // phase.  Atomics on the final root: extent, and the largest sum
            // (sums are >= 0, so their bit patterns order as the values do).
            // A position of this step still holds its bucketing record {0, 1}:
            // records change only on final roots, and sums only from (A') on.
            const bool fresh = q0 + k >= nd;
            const Rec8 rd = fresh ? Rec8{0.0f, 1} : rec8[d[k]];
            atomicAdd(&rec8[c[k]].size, rd.size);
            if (c[k] != pd[k]) st_state(sl.parent + d[k], c[k]);
            if (rd.w > 0.0f) atomicMax(reinterpret_cast<unsigned int*>(&rec8[c[k]].w), __float_as_uint(rd.w));
          }
          continue;
        }
        int32_t sz[kSLanes];
        double wd[kSLanes], wr[kSLanes];
#pragma unroll
        for (int k = 0; k < kSLanes; ++k) {
          if (d[k] < 0) continue;
          if constexpr (kLazy) {
            const Rec rd = sl.rec[d[k]];
            sz[k] = rd.size;
            wd[k] = rd.w;
            if constexpr (!kMaxOnly) wr[k] = sl.rec[c[k]].w;
          } else {
            sz[k] = ld_state(sl.size + d[k]);
          }
        }
#pragma unroll
        for (int k = 0; k < kSLanes; ++k) {
          if (d[k] < 0) continue;
          if constexpr (kLazy) atomicAdd(&sl.rec[c[k]].size, sz[k]);
          else atomicAdd(sl.size + c[k], sz[k]);
          if (c[k] != pd[k]) st_state(sl.parent + d[k], c[k]);
          if constexpr (kMaxOnly) {
            // sums are >= 0, so their bit patterns order as the values do
            atomicMax(reinterpret_cast<unsigned long long*>(&sl.rec[c[k]].w),
                      static_cast<unsigned long long>(__double_as_longlong(wd[k])));
          } else if constexpr (kLazy) {
            sl.rec[d[k]].w = wd[k] - wr[k];
          }
        }
      }
      if constexpr (kLazy) {
        if (tid == 0) {
          sNext = 0;
          sGrabA = 0;
        }
      }
      __syncthreads();
      TFGB_PHASE_MARK(3);
      if (tid == 0) {
        sNDead = 0;
        sGrabS = 0;  // read again only after two more barriers
      }
      if constexpr (kLazy) {
        // (A') every live root adds its component's increment once: the old
        // live roots that survived this step plus the new vertices that are
        // roots, compacted into the next list as they are visited
        const float HHl = sHH[i];
        const int32_t n_old = sNRoots;
        const int32_t n_cand = n_old + (s1 - s0);
        for (int32_t q0 = atomicAdd(&sGrabA, kALanes); q0 < n_cand; q0 = atomicAdd(&sGrabA, kALanes)) {
          int32_t c[kALanes];
          bool is_root[kALanes];
#pragma unroll
          for (int k = 0; k < kALanes; ++k) {
            const int32_t q = q0 + k;
            c[k] = (q >= n_cand) ? -1 : (q < n_old) ? cur_roots[q] : s0 + (q - n_old);
          }
          if constexpr (kR8) {
            // no thread writes a record in this phase but its own root's sum
#pragma unroll
            for (int k = 0; k < kALanes; ++k) is_root[k] = (c[k] >= 0) && (ld_state(sl.parent + c[k]) == c[k]);
#pragma unroll
            for (int k = 0; k < kALanes; ++k) {
              if (!is_root[k]) continue;
              const Rec8 rc = rec8[c[k]];
              rec8[c[k]].w = __fadd_rn(rc.w, increment(rc.size, E, e_mode, HHl));
            }
          } else {
#pragma unroll
            for (int k = 0; k < kALanes; ++k) is_root[k] = (c[k] >= 0) && (ld_state(sl.parent + c[k]) == c[k]);
            int32_t sz[kALanes];
            double w[kALanes];
#pragma unroll
            for (int k = 0; k < kALanes; ++k) {
              if (!is_root[k]) continue;
              const Rec rc = sl.rec[c[k]];
              sz[k] = rc.size;
              w[k] = rc.w;
            }
#pragma unroll
            for (int k = 0; k < kALanes; ++k)
              if (is_root[k]) sl.rec[c[k]].w = w[k] + static_cast<double>(increment(sz[k], E, e_mode, HHl));
          }
          const unsigned mask = __activemask();
          const int lane = tid & 31;
#pragma unroll
          for (int k = 0; k < kALanes; ++k) {
            const unsigned roots = __ballot_sync(mask, is_root[k]);
            if (roots) {
              const int leader = __ffs(roots) - 1;
              int base = 0;
              if (lane == leader) base = atomicAdd(&sNext, __popc(roots));
              base = __shfl_sync(mask, base, leader);
              if (is_root[k]) nxt_roots[base + __popc(roots & ((1u << lane) - 1u))] = c[k];
            }
          }
        }
        if constexpr (kR8) {
          // the next step's positions: read first by its union phase, after
          // this phase's barrier
          if (i + 1 < L)
            for (int32_t q = s1 + tid; q < sStart[i + 2]; q += nth) {
              sl.parent[q] = q;
              rec8[q] = Rec8{0.0f, 1};
            }
        }
        __syncthreads();
        if (tid == 0) sNRoots = sNext;
        int32_t* t_ = cur_roots;
        cur_roots = nxt_roots;
        nxt_roots = t_;
        TFGB_PHASE_MARK(4);
        TFGB_STEP_DONE();
        continue;
      }
      // (A) per-vertex increment, threshold order.  Each thread takes kALanes
      // positions per round and issues their loads together (the chain
      // parent -> root -> extent is latency-bound otherwise).
      const float HH = sHH[i];
      for (int32_t base = tid; base < s1; base += kALanes * nth) {
        int32_t pp[kALanes], rt[kALanes];
        float ac[kALanes];
#pragma unroll
        for (int k = 0; k < kALanes; ++k) {
          pp[k] = base + k * nth;
          if (pp[k] < s1) {
            rt[k] = ld_state(sl.parent + pp[k]);
            ac[k] = sl.acc[pp[k]];
          }
        }
        int32_t up[kALanes];
#pragma unroll
        for (int k = 0; k < kALanes; ++k)
          up[k] = (pp[k] < s1 && rt[k] != pp[k]) ? ld_state(sl.parent + rt[k]) : -1;
#pragma unroll
        for (int k = 0; k < kALanes; ++k) {
          if (up[k] >= 0 && up[k] != rt[k]) {
            rt[k] = find_root(sl.parent, up[k], a.err);
            st_state(sl.parent + pp[k], rt[k]);
          }
        }
        int32_t ext[kALanes];
#pragma unroll
        for (int k = 0; k < kALanes; ++k)
          if (pp[k] < s1) ext[k] = ld_state(sl.size + rt[k]);
#pragma unroll
        for (int k = 0; k < kALanes; ++k) {
          if (pp[k] < s1) {
            sl.acc[pp[k]] = __fadd_rn(ac[k], increment(ext[k], E, e_mode, HH));
            if (a.labels && i < a.label_cap) {
              const int32_t v = sl.order[pp[k]];
              a.labels[(int64_t)i * Vs + v] = sl.order[rt[k]];
              a.extents[(int64_t)i * Vs + v] = ext[k];
            }
          }
        }
      }
      __syncthreads();
      TFGB_PHASE_MARK(4);
    }

    // ---- 4. scale, reduce, write
    if constexpr (kMaxOnly) {
      float best = (n_act < Vs) ? __fmul_rn(0.0f, scale) : -INFINITY;
      const int32_t nr = sNRoots;
      for (int32_t q = tid; q < nr; q += nth)
        best = fmaxf(best, __fmul_rn(kR8 ? rec8[cur_roots[q]].w : __double2float_rn(sl.rec[cur_roots[q]].w), scale));
      best = block_max(best, sRed);
      if (tid == 0 && a.out_max) a.out_max[item] = (best == -INFINITY) ? 0.0f : best;
      __syncthreads();
      TFGB_PHASE_MARK(5);
      continue;
    }
    if constexpr (kLazy) {
      // resolve every active vertex: sum of potentials along its parent chain
      for (int32_t p = tid; p < n_act; p += nth) {
        double sum = sl.rec[p].w;
        int32_t c = p, l = sl.parent[p];
        for (int it = 0; l != c && it < kWalkLimit; ++it) {
          c = l;
          sum += sl.rec[c].w;
          l = sl.parent[c];
        }
        if (a.out_mode == 2 && omap) sum += static_cast<double>(omap[sl.order[p]]);
        sl.acc[p] = __double2float_rn(sum);
      }
      __syncthreads();
    }
    float best = (n_act < Vs) ? __fmul_rn(0.0f, scale) : -INFINITY;
    if (a.out_mode == 1 && omap) {
      for (int32_t v = tid; v < Vs; v += nth) {
        const uint32_t k = sl.key[v];
        const float t = (k == kInactiveKey) ? 0.0f : sl.acc[k & ((1u << kPosBits) - 1u)];
        float val = __fmul_rn(t, scale);
        if (vd) val = __fmul_rn(val, vd[v]);
        omap[v] = val;
        best = fmaxf(best, val);
      }
    } else {
      for (int32_t p = tid; p < n_act; p += nth) {
        const float t = sl.acc[p];
        if (a.out_mode == 2 && omap) omap[sl.order[p]] = t;
        float val = __fmul_rn(t, scale);
        if (vd) val = __fmul_rn(val, vd[sl.order[p]]);
        best = fmaxf(best, val);
      }
    }
    best = block_max(best, sRed);
    if (tid == 0 && a.out_max) a.out_max[item] = (best == -INFINITY) ? 0.0f : best;
    __syncthreads();
    TFGB_PHASE_MARK(5);
  }
}

// Maximum of +x and of -x over every (map, segment), finite values only:
// seg_max[(map * signs + sign) * n_seg + seg].  One block per (map, segment).
__global__ void __launch_bounds__(256) segment_max_kernel(const float* __restrict__ stats, int64_t map_stride,
                                                          int32_t signs, const int64_t* __restrict__ seg_off,
                                                          int32_t n_seg, float* __restrict__ seg_max) {
  __shared__ float red[2][8];
  const int64_t b = blockIdx.x;
  const int32_t seg = static_cast<int32_t>(b % n_seg);
  const int64_t map = b / n_seg;
  const float* x = stats + map * map_stride;
  float mp = -INFINITY, mn = -INFINITY;
  for (int64_t v = seg_off[seg] + threadIdx.x; v < seg_off[seg + 1]; v += blockDim.x) {
    const float xv = x[v];
    if (isfinite(xv)) {
      mp = fmaxf(mp, xv);
      mn = fmaxf(mn, -xv);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    mp = fmaxf(mp, __shfl_xor_sync(0xffffffffu, mp, o));
    mn = fmaxf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    red[0][w] = mp;
    red[1][w] = mn;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) {
      mp = fmaxf(mp, red[0][i]);
      mn = fmaxf(mn, red[1][i]);
    }
    seg_max[(map * signs) * n_seg + seg] = mp;
    if (signs == 2) seg_max[(map * signs + 1) * n_seg + seg] = mn;
  }
}

}  // namespace tfgb

// ---------------------------------------------------------------------------
// Handle and C-ABI
// ---------------------------------------------------------------------------
struct tfce_adjset {
  int device = 0;
  int32_t V = 0;
  int64_t D = 0;
  int32_t n_seg = 1;
  bool symmetric = true;
  int32_t vmax_seg = 0;
  std::vector<int64_t> seg_off;
  std::vector<float> H, E;
  int64_t* d_offsets = nullptr;
  uint32_t* d_indices = nullptr;
  int64_t* d_seg_off = nullptr;
  float* d_H = nullptr;
  float* d_E = nullptr;
  int32_t* d_ctrl = nullptr;  // [0] queue counter, [1] error word, [2] step count
  char* d_ws = nullptr;
  int64_t ws_slot = 0;
  int32_t ws_slots = 0;
  int32_t max_slots = 0;
  float* d_img = nullptr;
  float* d_enh = nullptr;
  int32_t run_cap = 0;
  int32_t accumulation = 0;  // 0: reference arithmetic, 1: per-component
  bool no_max_only = false;  // accumulation 2: the potential form for maxima-only launches too
  int32_t ctas_per_sm = TFGB_SWEEP_MINBLOCKS;  // sweep CTA shape of the per-component launches (3 or 2)
  int32_t* d_group = nullptr;  // threshold group of every segment, or NULL
  float* d_segmax = nullptr;   // segment maxima of the last grouped launch
  int64_t segmax_cap = 0;
  // Device buffers replaced by larger ones.  A launch captured into a CUDA
  // graph keeps the workspace pointer it was captured with, so a buffer is
  // never freed while the handle lives: it is retired here and freed by
  // tfce_adjset_destroy.  Growth is geometric, so the retired total stays
  // below the live buffer's size.
  std::vector<void*> retired;
  // Segments of uneven sizes: the segments by decreasing size, so items are
  // handed out largest segment first (every map of the largest segment, then
  // the next) and a launch does not end on a few long sweeps.  NULL when all
  // segments have the same size.
  int32_t* d_segrank = nullptr;
  std::mutex mu;
};

namespace {

int release(tfce_adjset* h) {
  if (!h) return TFCE_OK;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaSetDevice(h->device);
  cudaFree(h->d_offsets);
  cudaFree(h->d_indices);
  cudaFree(h->d_seg_off);
  cudaFree(h->d_H);
  cudaFree(h->d_E);
  cudaFree(h->d_ctrl);
  cudaFree(h->d_ws);
  cudaFree(h->d_img);
  cudaFree(h->d_enh);
  cudaFree(h->d_group);
  cudaFree(h->d_segmax);
  cudaFree(h->d_segrank);
  for (void* p : h->retired) cudaFree(p);
  h->retired.clear();
  cudaSetDevice(dev);
  return TFCE_OK;
}

int resident_slots(tfce_adjset* h) {
  if (h->max_slots) return TFCE_OK;
  int sms = 0, per_sm = 0;
  TFGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device));
  if (h->ctas_per_sm == 2)
    TFGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tfgb::tfce_sweep_kernel<false, true, true, 2>,
                                                            tfgb::kSweepThreads, tfgb::bitmap_bytes(h->vmax_seg)));
  else
    TFGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tfgb::tfce_sweep_kernel<false, false>,
                                                            tfgb::kSweepThreads, tfgb::bitmap_bytes(h->vmax_seg)));
  h->max_slots = std::max(1, sms * std::max(1, per_sm));
  // tuning knob: fewer CTAs in flight (smaller L2 working set)
  if (const char* env = std::getenv("TFCE_SWEEP_MAX_CTAS")) {
    const int cap = std::atoi(env);
    if (cap > 0) h->max_slots = std::min(h->max_slots, cap);
  }
  return TFCE_OK;
}

// One slot layout serves both accumulation modes (the per-component layout
// is the larger), so switching modes never replaces the workspace; a launch
// with more items than the workspace has slots replaces it by one at least
// twice as large (capped at the resident-slot count), retiring the old one.
int ensure_workspace(tfce_adjset* h, int32_t slots, bool lazy) {
  (void)lazy;
  const int64_t per = std::max(tfgb::slot_bytes_lazy(h->vmax_seg), tfgb::slot_bytes(h->vmax_seg));
  if (h->d_ws && h->ws_slots >= slots && h->ws_slot >= per) return TFCE_OK;
  const int32_t want = std::max(slots, std::min(h->max_slots, 2 * h->ws_slots));
  char* fresh = nullptr;
  TFGB_CUDA(cudaMalloc(&fresh, per * want));
  if (h->d_ws) h->retired.push_back(h->d_ws);
  h->d_ws = fresh;
  h->ws_slot = per;
  h->ws_slots = want;
  return TFCE_OK;
}

int launch_sweep(tfce_adjset* h, const float* stats, int64_t map_stride, int32_t n_maps,
                 int32_t signs, const float* vdensity, int32_t floor_zero, float* out_max,
                 float* out_maps, int32_t out_mode, int32_t* labels, int32_t* extents,
                 int32_t label_cap, cudaStream_t st, bool lazy) {
  const int64_t items64 = (int64_t)n_maps * signs * h->n_seg;
  TFGB_CHECK_ARG(items64 < (1LL << 31), "too many sweep items");
  const int32_t items = static_cast<int32_t>(items64);
  if (items == 0) return TFCE_OK;
  int rs = resident_slots(h);
  if (rs) return rs;
  const int32_t slots = std::min<int32_t>(items, h->max_slots);
  int rc = ensure_workspace(h, slots, lazy);
  if (rc) return rc;
  TFGB_CUDA(cudaMemsetAsync(h->d_ctrl, 0, sizeof(int32_t), st));  // queue counter only
  tfgb::SweepArgs a{};
  a.offsets = h->d_offsets;
  a.indices = h->d_indices;
  a.stats = stats;
  a.map_stride = map_stride;
  a.n_maps = n_maps;
  a.n_signs = signs;
  a.n_seg = h->n_seg;
  a.seg_off = h->d_seg_off;
  a.seg_H = h->d_H;
  a.seg_E = h->d_E;
  a.vdensity = vdensity;
  a.floor_zero = floor_zero;
  a.out_max = out_max;
  a.out_maps = out_maps;
  a.out_mode = out_mode;
  a.labels = labels;
  a.extents = extents;
  a.n_steps_out = labels ? h->d_ctrl + 2 : nullptr;
  a.label_cap = label_cap;
  a.ws = h->d_ws;
  a.ws_slot_bytes = h->ws_slot;
  a.vcap = h->vmax_seg;
  a.counter = h->d_ctrl;
  a.err = h->d_ctrl + 1;
  a.n_items = items;
  a.item_order = nullptr;
  a.seg_rank = h->d_segrank;
  const int bm = tfgb::bitmap_bytes(h->vmax_seg);
  a.bm_words = bm / 4;
  if (h->d_group) {
    const int64_t need = (int64_t)n_maps * signs * h->n_seg;
    if (h->segmax_cap < need) {
      const int64_t cap = std::max(need, 2 * h->segmax_cap);
      float* fresh = nullptr;
      TFGB_CUDA(cudaMalloc(&fresh, sizeof(float) * cap));
      if (h->d_segmax) h->retired.push_back(h->d_segmax);  // a captured launch may still use it
      h->d_segmax = fresh;
      h->segmax_cap = cap;
    }
    const int64_t blocks = (int64_t)n_maps * h->n_seg;
    TFGB_CHECK_ARG(blocks < (1LL << 31), "too many segment-max blocks");
    tfgb::segment_max_kernel<<<static_cast<unsigned>(blocks), 256, 0, st>>>(stats, map_stride, signs,
                                                                          h->d_seg_off, h->n_seg, h->d_segmax);
    TFGB_CUDA(cudaGetLastError());
    a.thr_group = h->d_group;
    a.seg_max = h->d_segmax;
  }
  // maxima only, no vertex weights: the per-component form without potentials
  const bool max_only = lazy && !vdensity && !out_maps && !labels && out_max && !h->no_max_only;
  const bool two = (h->ctas_per_sm == 2);
  if (max_only && two) tfgb::tfce_sweep_kernel<false, true, true, 2><<<slots, tfgb::kSweepThreads, bm, st>>>(a);
  else if (max_only) tfgb::tfce_sweep_kernel<false, true, true><<<slots, tfgb::kSweepThreads, bm, st>>>(a);
  else if (lazy && two) tfgb::tfce_sweep_kernel<false, true, false, 2><<<slots, tfgb::kSweepThreads, bm, st>>>(a);
  else if (lazy) tfgb::tfce_sweep_kernel<false, true><<<slots, tfgb::kSweepThreads, bm, st>>>(a);
  else tfgb::tfce_sweep_kernel<false, false><<<slots, tfgb::kSweepThreads, bm, st>>>(a);
  TFGB_CUDA(cudaGetLastError());
  return TFCE_OK;
}

// Reads and clears the sticky error word (synchronises the stream).
int check_device_error(tfce_adjset* h, cudaStream_t st, int32_t* steps) {
  int32_t ctrl[4];
  TFGB_CUDA(cudaMemcpyAsync(ctrl, h->d_ctrl, sizeof(ctrl), cudaMemcpyDeviceToHost, st));
  TFGB_CUDA(cudaStreamSynchronize(st));
  if (steps) *steps = ctrl[2];
  if (ctrl[1] != 0) TFGB_CUDA(cudaMemsetAsync(h->d_ctrl + 1, 0, sizeof(int32_t), st));
  return tfgb::map_dev_err(ctrl[1]);
}

int ensure_run_buffers(tfce_adjset* h, int32_t V) {
  if (h->run_cap >= V) return TFCE_OK;
  cudaFree(h->d_img);
  cudaFree(h->d_enh);
  h->d_img = h->d_enh = nullptr;
  h->run_cap = 0;
  TFGB_CUDA(cudaMalloc(&h->d_img, sizeof(float) * std::max(V, 1)));
  TFGB_CUDA(cudaMalloc(&h->d_enh, sizeof(float) * std::max(V, 1)));
  h->run_cap = V;
  return TFCE_OK;
}

}  // namespace

extern "C" {

int tfce_adjset_create(const int64_t* offsets, const int32_t* indices, int32_t n_vertices,
                       const int64_t* seg_offsets, int32_t n_seg, const float* H, const float* E,
                       tfce_adjset** out) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(out != nullptr, "out is NULL");
  *out = nullptr;
  TFGB_CHECK_ARG(n_vertices >= 0, "n_vertices < 0");
  TFGB_CHECK_ARG(offsets != nullptr, "offsets is NULL");
  TFGB_CHECK_ARG(H != nullptr && E != nullptr, "H/E is NULL");
  if (!seg_offsets) n_seg = 1;
  TFGB_CHECK_ARG(n_seg >= 1, "n_seg < 1");
  const int32_t V = n_vertices;
  TFGB_CHECK_ARG(offsets[0] == 0, "offsets[0] != 0");
  for (int32_t v = 0; v < V; ++v) TFGB_CHECK_ARG(offsets[v + 1] >= offsets[v], "offsets not monotone");
  const int64_t D = offsets[V];
  TFGB_CHECK_ARG(D == 0 || indices != nullptr, "indices is NULL");
  std::vector<int64_t> seg(n_seg + 1);
  if (seg_offsets) {
    for (int s = 0; s <= n_seg; ++s) seg[s] = seg_offsets[s];
    TFGB_CHECK_ARG(seg[0] == 0 && seg[n_seg] == V, "segment offsets must span [0, V]");
    for (int s = 0; s < n_seg; ++s) TFGB_CHECK_ARG(seg[s + 1] >= seg[s], "segment offsets not monotone");
  } else {
    seg[0] = 0;
    seg[1] = V;
  }
  std::vector<int32_t> seg_of(V);
  int32_t vmax = 1;
  for (int s = 0; s < n_seg; ++s) {
    const int64_t len = seg[s + 1] - seg[s];
    TFGB_CHECK_ARG(len <= tfgb::kMaxSegVertices, "segment larger than 2^24-1 vertices");
    vmax = std::max<int32_t>(vmax, static_cast<int32_t>(len));
    for (int64_t v = seg[s]; v < seg[s + 1]; ++v) seg_of[v] = s;
  }
  for (int s = 0; s < n_seg; ++s) {
    TFGB_CHECK_ARG(std::isfinite(H[s]) && std::isfinite(E[s]), "H/E must be finite");
  }

  // Clean the lists: validate, drop self entries, mark entries whose reverse
  // is missing.  Neighbour order inside a list never changes the partition.
  std::vector<int64_t> off(V + 1, 0);
  std::vector<int32_t> idx;
  idx.reserve(static_cast<size_t>(D));
  for (int32_t v = 0; v < V; ++v) {
    for (int64_t e = offsets[v]; e < offsets[v + 1]; ++e) {
      const int32_t b = indices[e];
      if (b < 0 || b >= V) {
        tfgb::set_error("adjacency entry %d of vertex %d outside [0, %d)", b, v, V);
        return TFCE_EINVAL;
      }
      if (seg_of[b] != seg_of[v]) {
        tfgb::set_error("adjacency entry %d of vertex %d crosses segments", b, v);
        return TFCE_EINVAL;
      }
      if (b != v) idx.push_back(b);
    }
    off[v + 1] = static_cast<int64_t>(idx.size());
  }
  for (int32_t v = 0; v < V; ++v) std::sort(idx.begin() + off[v], idx.begin() + off[v + 1]);
  std::vector<uint32_t> packed(idx.size());
  bool symmetric = true;
  for (int32_t v = 0; v < V; ++v) {
    for (int64_t e = off[v]; e < off[v + 1]; ++e) {
      const int32_t b = idx[e];
      const bool rev = std::binary_search(idx.begin() + off[b], idx.begin() + off[b + 1], v);
      packed[e] = static_cast<uint32_t>(b) | (rev ? 0u : tfgb::kOneWay);
      symmetric = symmetric && rev;
    }
  }

  tfce_adjset* h = new tfce_adjset();
  cudaGetDevice(&h->device);
  h->V = V;
  h->D = static_cast<int64_t>(packed.size());
  h->n_seg = n_seg;
  h->symmetric = symmetric;
  h->vmax_seg = vmax;
  h->seg_off = seg;
  h->H.assign(H, H + n_seg);
  h->E.assign(E, E + n_seg);
  auto fail = [&](int rc) {
    release(h);
    delete h;
    return rc;
  };
#define TFGB_CUDA_H(call)                                                           \
  do {                                                                              \
    cudaError_t _e = (call);                                                        \
    if (_e != cudaSuccess) {                                                        \
      tfgb::set_error("%s: %s", #call, cudaGetErrorString(_e));                     \
      return fail(_e == cudaErrorMemoryAllocation ? TFCE_ENOMEM : TFCE_EDEVICE);    \
    }                                                                               \
  } while (0)
  TFGB_CUDA_H(cudaMalloc(&h->d_offsets, sizeof(int64_t) * (V + 1)));
  TFGB_CUDA_H(cudaMalloc(&h->d_indices, sizeof(uint32_t) * std::max<size_t>(1, packed.size())));
  TFGB_CUDA_H(cudaMalloc(&h->d_seg_off, sizeof(int64_t) * (n_seg + 1)));
  TFGB_CUDA_H(cudaMalloc(&h->d_H, sizeof(float) * n_seg));
  TFGB_CUDA_H(cudaMalloc(&h->d_E, sizeof(float) * n_seg));
  TFGB_CUDA_H(cudaMalloc(&h->d_ctrl, sizeof(int32_t) * 4));
  TFGB_CUDA_H(cudaMemset(h->d_ctrl, 0, sizeof(int32_t) * 4));
  TFGB_CUDA_H(cudaMemcpy(h->d_offsets, off.data(), sizeof(int64_t) * (V + 1), cudaMemcpyHostToDevice));
  if (!packed.empty())
    TFGB_CUDA_H(cudaMemcpy(h->d_indices, packed.data(), sizeof(uint32_t) * packed.size(),
                           cudaMemcpyHostToDevice));
  TFGB_CUDA_H(cudaMemcpy(h->d_seg_off, seg.data(), sizeof(int64_t) * (n_seg + 1), cudaMemcpyHostToDevice));
  TFGB_CUDA_H(cudaMemcpy(h->d_H, H, sizeof(float) * n_seg, cudaMemcpyHostToDevice));
  TFGB_CUDA_H(cudaMemcpy(h->d_E, E, sizeof(float) * n_seg, cudaMemcpyHostToDevice));
  bool uneven = false;
  for (int s = 0; s + 1 < n_seg; ++s) uneven = uneven || (seg[s + 1] - seg[s] != seg[s + 2] - seg[s + 1]);
  if (uneven) {
    std::vector<int32_t> rank(n_seg);
    for (int32_t s = 0; s < n_seg; ++s) rank[s] = s;
    std::stable_sort(rank.begin(), rank.end(),
                     [&](int32_t x, int32_t y) { return seg[x + 1] - seg[x] > seg[y + 1] - seg[y]; });
    TFGB_CUDA_H(cudaMalloc(&h->d_segrank, sizeof(int32_t) * n_seg));
    TFGB_CUDA_H(cudaMemcpy(h->d_segrank, rank.data(), sizeof(int32_t) * n_seg, cudaMemcpyHostToDevice));
  }
#undef TFGB_CUDA_H
  *out = h;
  return TFCE_OK;
}

void tfce_adjset_destroy(tfce_adjset* h) {
  if (!h) return;
  release(h);
  delete h;
}

int tfce_adjset_set_params(tfce_adjset* h, const float* H, const float* E) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(h && H && E, "NULL argument");
  std::lock_guard<std::mutex> lk(h->mu);
  for (int s = 0; s < h->n_seg; ++s)
    TFGB_CHECK_ARG(std::isfinite(H[s]) && std::isfinite(E[s]), "H/E must be finite");
  h->H.assign(H, H + h->n_seg);
  h->E.assign(E, E + h->n_seg);
  TFGB_CUDA(cudaMemcpy(h->d_H, H, sizeof(float) * h->n_seg, cudaMemcpyHostToDevice));
  TFGB_CUDA(cudaMemcpy(h->d_E, E, sizeof(float) * h->n_seg, cudaMemcpyHostToDevice));
  return TFCE_OK;
}

int tfce_adjset_is_symmetric(const tfce_adjset* h) { return (h && h->symmetric) ? 1 : 0; }

int tfce_adjset_set_sweep_shape(tfce_adjset* h, int32_t ctas_per_sm) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(h != nullptr, "handle is NULL");
  TFGB_CHECK_ARG(ctas_per_sm == 2 || ctas_per_sm == 3, "ctas_per_sm must be 2 or 3");
  std::lock_guard<std::mutex> lk(h->mu);
  if (h->ctas_per_sm != ctas_per_sm) {
    h->ctas_per_sm = ctas_per_sm;
    h->max_slots = 0;  // recomputed for the new shape at the next launch
  }
  return TFCE_OK;
}

int tfce_adjset_set_threshold_groups(tfce_adjset* h, const int32_t* group) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(h != nullptr, "handle is NULL");
  std::lock_guard<std::mutex> lk(h->mu);
  if (!group) {
    cudaFree(h->d_group);
    h->d_group = nullptr;
    return TFCE_OK;
  }
  for (int s = 0; s < h->n_seg; ++s) TFGB_CHECK_ARG(group[s] >= 0 && group[s] < h->n_seg, "group id outside [0, n_seg)");
  if (!h->d_group) TFGB_CUDA(cudaMalloc(&h->d_group, sizeof(int32_t) * h->n_seg));
  TFGB_CUDA(cudaMemcpy(h->d_group, group, sizeof(int32_t) * h->n_seg, cudaMemcpyHostToDevice));
  return TFCE_OK;
}

int tfce_adjset_set_accumulation(tfce_adjset* h, int32_t mode) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(h != nullptr, "handle is NULL");
  TFGB_CHECK_ARG(mode >= 0 && mode <= 2, "mode must be 0 (reference), 1 (per-component) or 2 (per-component, "
                                          "potentials kept)");
  std::lock_guard<std::mutex> lk(h->mu);
  h->accumulation = mode == 0 ? 0 : 1;
  h->no_max_only = (mode == 2);
  return TFCE_OK;
}

int tfce_adjset_run(tfce_adjset* h, const float* image, float* enhn, int32_t n_vertices) {
  return tfce_adjset_run_labels(h, image, enhn, n_vertices, nullptr, nullptr, 0, nullptr);
}

int tfce_adjset_run_labels(tfce_adjset* h, const float* image, float* enhn, int32_t n_vertices,
                           int32_t* labels, int32_t* extents, int32_t max_steps,
                           int32_t* n_steps) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(h != nullptr, "handle is NULL");
  TFGB_CHECK_ARG(image != nullptr && enhn != nullptr, "image/enhn is NULL");
  TFGB_CHECK_ARG(n_vertices == h->V, "array length differs from the adjacency set's vertex count");
  TFGB_CHECK_ARG(h->n_seg == 1 || labels == nullptr, "label recording needs a one-segment handle");
  TFGB_CHECK_ARG(labels == nullptr || (extents != nullptr && max_steps > 0), "labels need extents/max_steps");
  std::lock_guard<std::mutex> lk(h->mu);
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != h->device) TFGB_CUDA(cudaSetDevice(h->device));
  const int32_t V = h->V;
  int rc = ensure_run_buffers(h, V);
  int32_t *d_lab = nullptr, *d_ext = nullptr;
  if (rc == TFCE_OK && V > 0) {
    cudaStream_t st = nullptr;
    const size_t lab_bytes = sizeof(int32_t) * (size_t)max_steps * V;
    do {
      if (labels) {
        if (cudaMalloc(&d_lab, lab_bytes) != cudaSuccess || cudaMalloc(&d_ext, lab_bytes) != cudaSuccess) {
          tfgb::set_error("label buffers: out of device memory");
          rc = TFCE_ENOMEM;
          break;
        }
        if (cudaMemset(d_lab, 0xff, lab_bytes) != cudaSuccess || cudaMemset(d_ext, 0, lab_bytes) != cudaSuccess) {
          rc = TFCE_EDEVICE;
          break;
        }
      }
      if (cudaMemcpy(h->d_img, image, sizeof(float) * V, cudaMemcpyHostToDevice) != cudaSuccess ||
          cudaMemcpy(h->d_enh, enhn, sizeof(float) * V, cudaMemcpyHostToDevice) != cudaSuccess) {
        tfgb::set_error("host->device copy failed");
        rc = TFCE_EDEVICE;
        break;
      }
      rc = launch_sweep(h, h->d_img, V, 1, 1, nullptr, 0, nullptr, h->d_enh, 2, d_lab, d_ext,
                        max_steps, st, false);
      if (rc) break;
      int32_t steps = 0;
      rc = check_device_error(h, st, &steps);
      if (rc) break;
      if (cudaMemcpy(enhn, h->d_enh, sizeof(float) * V, cudaMemcpyDeviceToHost) != cudaSuccess) {
        tfgb::set_error("device->host copy failed");
        rc = TFCE_EDEVICE;
        break;
      }
      if (labels) {
        const int32_t keep = std::min(steps, max_steps);
        if (cudaMemcpy(labels, d_lab, sizeof(int32_t) * (size_t)keep * V, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(extents, d_ext, sizeof(int32_t) * (size_t)keep * V, cudaMemcpyDeviceToHost) != cudaSuccess) {
          rc = TFCE_EDEVICE;
          break;
        }
        if (steps > max_steps) {
          tfgb::set_error("label buffer holds %d steps, sweep used %d", max_steps, steps);
          rc = TFCE_ERANGE;
        }
      }
      if (n_steps) *n_steps = steps;
    } while (0);
  }
  cudaFree(d_lab);
  cudaFree(d_ext);
  if (dev != h->device) cudaSetDevice(dev);
  return rc;
}

int tfce_sweep_batch(tfce_adjset* h, const float* stats, int64_t map_stride, int32_t n_maps,
                     int32_t signs, const float* vdensity, int32_t floor_zero, float* out_max,
                     float* out_maps, int32_t out_mode, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(h != nullptr, "handle is NULL");
  TFGB_CHECK_ARG(n_maps >= 0, "n_maps < 0");
  TFGB_CHECK_ARG(signs == 1 || signs == 2, "signs must be 1 or 2");
  TFGB_CHECK_ARG(n_maps == 0 || stats != nullptr, "stats is NULL");
  TFGB_CHECK_ARG(map_stride >= h->V, "map_stride < V");
  TFGB_CHECK_ARG(out_mode >= 0 && out_mode <= 2, "out_mode must be 0, 1 or 2");
  TFGB_CHECK_ARG(out_mode == 0 || out_maps != nullptr, "out_maps is NULL");
  TFGB_CHECK_ARG(out_max != nullptr || out_mode != 0, "nothing to write");
  std::lock_guard<std::mutex> lk(h->mu);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = launch_sweep(h, stats, map_stride, n_maps, signs, vdensity, floor_zero, out_max,
                        out_maps, out_mode, nullptr, nullptr, 0, st, h->accumulation == 1);
  return rc;
}

#ifdef TFGB_PHASE_PROFILE
// Debug-only export: per-phase cycle sums since the last call (then cleared).
int tfce_debug_step_cycles(unsigned long long* out128) {
  TFGB_CUDA(cudaDeviceSynchronize());
  TFGB_CUDA(cudaMemcpyFromSymbol(out128, tfgb::g_step_cycles, 128 * sizeof(unsigned long long)));
  unsigned long long z[128] = {0};
  TFGB_CUDA(cudaMemcpyToSymbol(tfgb::g_step_cycles, z, sizeof(z)));
  return TFCE_OK;
}

int tfce_debug_phase_cycles(unsigned long long* out16) {
  TFGB_CUDA(cudaDeviceSynchronize());
  TFGB_CUDA(cudaMemcpyFromSymbol(out16, tfgb::g_phase_cycles, 8 * sizeof(unsigned long long)));
  TFGB_CUDA(cudaMemcpyFromSymbol(out16 + 8, tfgb::g_dbg_counts, 8 * sizeof(unsigned long long)));
  unsigned long long z[8] = {0};
  TFGB_CUDA(cudaMemcpyToSymbol(tfgb::g_phase_cycles, z, sizeof(z)));
  TFGB_CUDA(cudaMemcpyToSymbol(tfgb::g_dbg_counts, z, sizeof(z)));
  return TFCE_OK;
}
#endif

// Error word of the last batched sweep on this handle (synchronises `stream`).
int tfce_sweep_resident_slots(tfce_adjset* h, int32_t* slots) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(h != nullptr && slots != nullptr, "NULL pointer");
  std::lock_guard<std::mutex> lk(h->mu);
  const int rc = resident_slots(h);
  if (rc) return rc;
  *slots = h->max_slots;
  return TFCE_OK;
}

int tfce_sweep_status(tfce_adjset* h, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(h != nullptr, "handle is NULL");
  std::lock_guard<std::mutex> lk(h->mu);
  return check_device_error(h, static_cast<cudaStream_t>(stream), nullptr);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free batched sweep.
//
// For callers that cannot allocate device memory while they run the sweep:
// programs whose device memory is reserved up front by another allocator (a
// framework's caching allocator holding the whole GPU), real-time loops that
// must keep a fixed footprint, and hosts that cannot afford the device-wide
// synchronisation cudaFree implies.  The sweep's scratch (the per-CTA union-
// find workspace and the queue/error words) lives in the file-scope array
// below instead of in cudaMalloc'd memory.  Every process that loads this
// library holds these 64 MiB on every GPU it uses, until it exits.
// ---------------------------------------------------------------------------
namespace tfgb {

constexpr int64_t kNoAllocScratchBytes = 64LL << 20;   // 64 MiB
constexpr int64_t kNoAllocCtrlBytes = 256;              // queue counter, error word
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct NoAllocDevice {
  void* scratch = nullptr;  // device address of g_noalloc_scratch in the current context
  int max_slots = 0;        // resident CTAs of the checked kernel
};

std::mutex g_noalloc_mu;
int g_noalloc_slots[128];  // resident CTAs per device ordinal (0 = not yet queried)

// Largest segment one workspace slot of the static scratch can hold.
int32_t noalloc_max_segment() {
  int64_t lo = 1, hi = kMaxSegVertices;
  while (lo < hi) {  // largest v with slot_bytes(v) <= scratch - ctrl
    const int64_t mid = (lo + hi + 1) / 2;
    if (slot_bytes(static_cast<int32_t>(mid)) <= kNoAllocScratchBytes - kNoAllocCtrlBytes) lo = mid;
    else hi = mid - 1;
  }
  return static_cast<int32_t>(lo);
}

// Set-up of every call, with the caller's device current: the host-side name
// of the array is not a device address, so its device address in the current
// context is looked up with cudaGetSymbolAddress (cheap; looked up on every
// call, so a context re-created after cudaDeviceReset is served correctly).
// The resident-CTA count is queried once per device ordinal.
int noalloc_setup(int dev, NoAllocDevice* out) {
  if (dev < 0 || dev >= 128) {
    set_error("device ordinal %d out of range", dev);
    return TFCE_EINVAL;
  }
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || p == nullptr) {
    set_error("cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    return TFCE_EDEVICE;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_slots[dev]) {
    int sms = 0, per_sm = 0;
    TFGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    TFGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tfce_sweep_kernel<true, false>,
                                                            kSweepThreads, 0));
    g_noalloc_slots[dev] = std::max(1, sms * std::max(1, per_sm));
  }
  out->scratch = p;
  out->max_slots = g_noalloc_slots[dev];
  return TFCE_OK;
}

}  // namespace tfgb

extern "C" int tfce_sweep_batch_noalloc(const int64_t* offsets, const int32_t* indices,
                                        int32_t n_vertices, int64_t n_entries,
                                        const int64_t* seg_offsets, int32_t n_seg,
                                        int32_t max_segment_vertices, const float* H,
                                        const float* E, const float* stats, int64_t map_stride,
                                        int32_t n_maps, int32_t signs, const float* vdensity,
                                        int32_t floor_zero, float* out_max, void* stream) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(offsets && seg_offsets && H && E && out_max, "NULL pointer");
  TFGB_CHECK_ARG(n_entries == 0 || indices != nullptr, "indices is NULL");
  TFGB_CHECK_ARG(n_vertices >= 0 && n_entries >= 0 && n_seg >= 1, "bad sizes");
  TFGB_CHECK_ARG(n_maps >= 0, "n_maps < 0");
  TFGB_CHECK_ARG(n_maps == 0 || stats != nullptr, "stats is NULL");
  TFGB_CHECK_ARG(signs == 1 || signs == 2, "signs must be 1 or 2");
  TFGB_CHECK_ARG(map_stride >= n_vertices, "map_stride < n_vertices");
  TFGB_CHECK_ARG(max_segment_vertices >= 1, "max_segment_vertices < 1");
  const int32_t cap = tfgb::noalloc_max_segment();
  if (max_segment_vertices > cap) {
    tfgb::set_error("segments of %d vertices exceed the static scratch: at most %d vertices per "
                    "segment (64 MiB)", max_segment_vertices, cap);
    return TFCE_ERANGE;
  }
  const int64_t items64 = (int64_t)n_maps * signs * n_seg;
  TFGB_CHECK_ARG(items64 < (1LL << 31), "too many sweep items");
  const int32_t items = static_cast<int32_t>(items64);
  if (items == 0) return TFCE_OK;
  int dev = 0;
  TFGB_CUDA(cudaGetDevice(&dev));
  tfgb::NoAllocDevice nd;
  int rc = tfgb::noalloc_setup(dev, &nd);
  if (rc) return rc;
  const int64_t per_slot = tfgb::slot_bytes(max_segment_vertices);
  const int64_t fit = (tfgb::kNoAllocScratchBytes - tfgb::kNoAllocCtrlBytes) / per_slot;
  const int32_t slots = static_cast<int32_t>(std::min<int64_t>({(int64_t)items, fit, (int64_t)nd.max_slots}));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* base = static_cast<char*>(nd.scratch);
  int32_t* ctrl = reinterpret_cast<int32_t*>(base);
  // the array keeps the previous call's contents: the queue counter and the
  // error word must start at zero; the workspace slots are rebuilt per item
  TFGB_CUDA(cudaMemsetAsync(ctrl, 0, 4 * sizeof(int32_t), st));
  tfgb::SweepArgs a{};
  a.offsets = offsets;
  a.indices = reinterpret_cast<const uint32_t*>(indices);
  a.stats = stats;
  a.map_stride = map_stride;
  a.n_maps = n_maps;
  a.n_signs = signs;
  a.n_seg = n_seg;
  a.seg_off = seg_offsets;
  a.seg_H = H;
  a.seg_E = E;
  a.vdensity = vdensity;
  a.floor_zero = floor_zero;
  a.out_max = out_max;
  a.out_maps = nullptr;
  a.out_mode = 0;
  a.ws = base + tfgb::kNoAllocCtrlBytes;
  a.ws_slot_bytes = per_slot;
  a.vcap = max_segment_vertices;
  a.counter = ctrl;
  a.err = ctrl + 1;
  a.n_items = items;
  a.n_vertices = n_vertices;
  a.n_entries = n_entries;
  tfgb::tfce_sweep_kernel<true, false><<<slots, tfgb::kSweepThreads, 0, st>>>(a);
  TFGB_CUDA(cudaGetLastError());
  int32_t hctrl[2] = {0, 0};
  TFGB_CUDA(cudaMemcpyAsync(hctrl, ctrl, sizeof(hctrl), cudaMemcpyDeviceToHost, st));
  TFGB_CUDA(cudaStreamSynchronize(st));
  return tfgb::map_dev_err(hctrl[1]);
}
