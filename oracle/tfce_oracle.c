/*
 * ORACLE -- test infrastructure, not product code.
 *
 * CPU restatement of the reference's single-map TFCE sweep
 * (tfce_mediation/lib/fast_tfce.hpp:11-95, called through
 * tfce_mediation/tfce.pyx:44-45 with minT = 0, deltaT = 0).  Only the test
 * suite, the smoke check and the CPU-baseline leg of bench.py load this file's
 * shared library; the product path never does.
 *
 * Semantics restated (same arithmetic, own data structures):
 *   - vertices are visited by value, descending            (fast_tfce.hpp:27-30)
 *     ties are broken by ascending vertex index (the reference's std::sort is
 *     unstable, so its tie order is unspecified; only asymmetric adjacency
 *     lists can observe it);
 *   - maxT = largest value, dT = maxT / 100 in float        (:32-36)
 *   - thresholds T = maxT, maxT-dT, ... while T >= 0, by repeated float
 *     subtraction                                           (:39)
 *   - a vertex becomes active when value > T (strict) and is unioned with
 *     every listed neighbour that became active before it   (:41-64)
 *   - HH = powf(T, H); every active vertex receives
 *     (float)(pow((double)size, (double)E) * HH) where size is the extent of
 *     its component, accumulated into enhn in threshold order (:70-84)
 * Non-finite values are never activated and do not take part in maxT (the
 * reference's comparator is not a strict weak order for NaN).
 * A map whose maximum is <= 0 gets no increments (the reference never ends
 * its loop when the maximum is exactly 0, because dT is then 0).
 *
 * The union-find here (union by smaller index of the first-activated root,
 * path halving) replaces the reference's list-splicing disjoint sets; the
 * partition after every threshold is identical by construction.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_MAX_STEPS 4096

typedef struct {
  float v;
  int32_t i;
} vk_t;

static int cmp_desc(const void* pa, const void* pb) {
  const vk_t* a = (const vk_t*)pa;
  const vk_t* b = (const vk_t*)pb;
  if (a->v > b->v) return -1;
  if (a->v < b->v) return 1;
  return (a->i < b->i) ? -1 : (a->i > b->i);
}

static int32_t uf_find(int32_t* parent, int32_t x) {
  while (parent[x] != x) {
    parent[x] = parent[parent[x]];
    x = parent[x];
  }
  return x;
}

/* Threshold table by the reference's float recurrence.  Returns the number of
 * steps (0 when maxT <= 0 or not finite). */
int oracle_threshold_table(float maxT, float* T_out, int cap) {
  if (!(maxT > 0.0f) || !isfinite(maxT)) return 0;
  volatile float dT = maxT / 100;
  int n = 0;
  for (volatile float T = maxT; T >= 0.0f; T -= dT) {
    if (n >= cap) return -1;
    T_out[n++] = T;
  }
  return n;
}

/*
 * One TFCE sweep.  offsets/indices: CSR adjacency (entry b in the list of a
 * means the reference's adjacencyList[a] contains b).  enhn is accumulated
 * into, as the reference does.  Optional instrumentation:
 *   labels (n_steps x V): root vertex id of each vertex's component after the
 *   insertions of each threshold, -1 when inactive;
 *   extents (n_steps x V): size of that component, 0 when inactive.
 * Returns the number of thresholds processed, or -1 on error.
 */
/* HH at threshold T.  hh_mode 0: powf(T, H), what the reference computes
 * (fast_tfce.hpp:70).  hh_mode 1: the correctly rounded power -- T*T for
 * H == 2, else the double power rounded once -- which is what the device
 * computes; the two differ only where the libm powf is off by one ulp. */
static float oracle_hh(float T, float H, int hh_mode) {
  if (hh_mode == 0) return powf(T, H);
  if (H == 2.0f) return T * T;
  if (H == 1.0f) return T;
  return (float)pow((double)T, (double)H);
}

int oracle_tfce_mode(float H, float E, int32_t V, const int64_t* offsets,
                     const int32_t* indices, const float* image, float* enhn,
                     int32_t* labels, int32_t* extents, int max_steps, int hh_mode);

int oracle_tfce(float H, float E, int32_t V, const int64_t* offsets,
                const int32_t* indices, const float* image, float* enhn,
                int32_t* labels, int32_t* extents, int max_steps) {
  return oracle_tfce_mode(H, E, V, offsets, indices, image, enhn, labels, extents, max_steps, 0);
}

int oracle_tfce_mode(float H, float E, int32_t V, const int64_t* offsets,
                     const int32_t* indices, const float* image, float* enhn,
                     int32_t* labels, int32_t* extents, int max_steps, int hh_mode) {
  if (V <= 0) return 0;
  vk_t* keys = (vk_t*)malloc(sizeof(vk_t) * (size_t)V);
  int32_t* rank = (int32_t*)malloc(sizeof(int32_t) * (size_t)V);
  int32_t* parent = (int32_t*)malloc(sizeof(int32_t) * (size_t)V);
  int32_t* size = (int32_t*)malloc(sizeof(int32_t) * (size_t)V);
  int32_t* act = (int32_t*)malloc(sizeof(int32_t) * (size_t)V);
  float* T = (float*)malloc(sizeof(float) * ORACLE_MAX_STEPS);
  int32_t nv = 0;
  float maxT = -INFINITY;
  for (int32_t i = 0; i < V; ++i) {
    if (isfinite(image[i])) {
      keys[nv].v = image[i];
      keys[nv].i = i;
      if (image[i] > maxT) maxT = image[i];
      ++nv;
    }
    rank[i] = INT32_MAX;
  }
  qsort(keys, (size_t)nv, sizeof(vk_t), cmp_desc);
  for (int32_t r = 0; r < nv; ++r) rank[keys[r].i] = r;
  int L = (nv > 0) ? oracle_threshold_table(maxT, T, ORACLE_MAX_STEPS) : 0;
  if (L < 0) goto fail;
  if (max_steps >= 0 && L > max_steps) goto fail;

  int32_t j = 0, n_act = 0;
  for (int s = 0; s < L; ++s) {
    const float Ts = T[s];
    while (j < nv && keys[j].v > Ts) {
      const int32_t v = keys[j].i;
      parent[v] = v;
      size[v] = 1;
      act[n_act++] = v;
      for (int64_t e = offsets[v]; e < offsets[v + 1]; ++e) {
        const int32_t a = indices[e];
        if (a < 0 || a >= V) continue;
        if (rank[a] >= j) continue; /* not inserted before v */
        int32_t ra = uf_find(parent, a), rv = uf_find(parent, v);
        if (ra == rv) continue;
        /* keep the earlier-activated root (smaller rank) */
        if (rank[ra] < rank[rv]) {
          parent[rv] = ra;
          size[ra] += size[rv];
        } else {
          parent[ra] = rv;
          size[rv] += size[ra];
        }
      }
      ++j;
    }
    const float HH = oracle_hh(Ts, H, hh_mode);
    if (labels) for (int32_t u = 0; u < V; ++u) labels[(int64_t)s * V + u] = -1;
    if (extents) for (int32_t u = 0; u < V; ++u) extents[(int64_t)s * V + u] = 0;
    for (int32_t q = 0; q < n_act; ++q) {
      const int32_t u = act[q];
      const int32_t r = uf_find(parent, u);
      const float inc = (float)(pow((double)size[r], (double)E) * (double)HH);
      enhn[u] += inc;
      if (labels) labels[(int64_t)s * V + u] = r;
      if (extents) extents[(int64_t)s * V + u] = size[r];
    }
  }
  free(keys); free(rank); free(parent); free(size); free(act); free(T);
  return L;
fail:
  free(keys); free(rank); free(parent); free(size); free(act); free(T);
  return -1;
}

/*
 * Batched helper for the CPU baseline: n_maps maps of V values (row stride
 * V), each swept with the given sign, scaled the way
 * tfce_mediation/pyfunc.py:116-118 does: TFCE * (max(stat)/100) * vdensity,
 * and reduced to its maximum.  vdensity may be NULL (weight 1).
 * floor_zero != 0 means the map was scattered into a zero-filled array, so
 * its maximum is at least 0.
 */
int oracle_tfce_max_batch(float H, float E, int32_t V, const int64_t* offsets,
                          const int32_t* indices, const float* maps,
                          int32_t n_maps, float sign, const float* vdensity,
                          int floor_zero, float* out_max, int hh_mode) {
  float* img = (float*)malloc(sizeof(float) * (size_t)V);
  float* enh = (float*)malloc(sizeof(float) * (size_t)V);
  for (int32_t m = 0; m < n_maps; ++m) {
    float mx = floor_zero ? 0.0f : -INFINITY;
    for (int32_t i = 0; i < V; ++i) {
      img[i] = sign * maps[(int64_t)m * V + i];
      enh[i] = 0.0f;
      if (isfinite(img[i]) && img[i] > mx) mx = img[i];
    }
    if (oracle_tfce_mode(H, E, V, offsets, indices, img, enh, NULL, NULL, -1, hh_mode) < 0) {
      free(img); free(enh);
      return -1;
    }
    const float scale = mx / 100.0f;
    float best = -INFINITY;
    for (int32_t i = 0; i < V; ++i) {
      float val = enh[i] * scale;
      if (vdensity) val = val * vdensity[i];
      if (isfinite(val) && val > best) best = val;
    }
    out_max[m] = best;
  }
  free(img); free(enh);
  return 0;
}
