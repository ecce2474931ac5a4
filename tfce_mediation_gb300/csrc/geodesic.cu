// Exact geodesic distance lists on one GB300 (sm_103a).
//
// For every source vertex i of a triangle mesh: the vertices j within a
// geodesic radius and their exact distances.  This replaces the reference's
// tfce_mediation/adjacency.pyx:44-106 (compute, compute_distance_parallel),
// which runs its exact geodesic library (tfce_mediation/lib/geodesic,
// Kirsanov's implementation of Mitchell-Mount-Papadimitriou) one source at a
// time on one CPU core and then queries every vertex j > i.
//
// Method: window propagation (Chen and Han, with the end-vertex filter of Xin
// and Wang, ACM TOG 28(4), 2009), in double precision from the float32
// coordinates.  A window is an interval [b0, b1] of a face edge, the unfolded
// image s = (sx, sy) of its (pseudo-)source in that edge's 2-D frame (edge from
// (0, 0) to (L, 0), the face it enters on the +y side, s at y < 0) and the
// distance sigma from the source to s.  Crossing the face, a window reaches
// the third vertex C when the line s -> C meets the interval, and splits into
// at most two children on the other edges, re-expressed in the frames of the
// faces beyond them.  Vertices whose total angle exceeds 2 pi - 1e-5, and
// boundary vertices, are pseudo-sources (the reference's rule,
// geodesic_mesh.h:335-344).  A window is dropped when an end vertex of its
// edge gives a shorter path to every point of the interval, or when it lies
// beyond the radius.
//
// GPU mapping: sources are independent.  geodesic_warp_kernel gives each
// source a warp: the keys of its pending windows and pseudo-sources and its
// table of reached vertices sit in the warp's shared memory, and each round
// the 32 lanes propagate the items within one edge length of the smallest
// pending key (the filters are sound in any order, so the distances are the
// same exact ones).  A source that outgrows the warp's queue or table runs
// again in geodesic_lists_kernel, one thread per source with a binary heap
// and a table in global scratch laid out [slot][thread], with four and then
// sixteen times the room.  The mesh tables are read-only face-edge records
// shared by all (L2-resident).  Every loop is bounded.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <numeric>
#include <vector>

#include "common.cuh"

namespace tfgb {
namespace geo {

constexpr int kThreads = 128;
constexpr int64_t kIterLimit = int64_t(1) << 22;  // heap pops / rounds per source

// Everything a window crossing needs about local edge e of face f, in one
// 64-byte record, so that a crossing is a few dependent loads, not a dozen.
struct alignas(16) FaceEdge {
  double len;      // |f_e f_{e+1}|
  double inv_len;  // 1 / len
  double cx, cy;   // the third vertex f_{e+2} in this edge's frame (cy > 0)
  int32_t a, b, c; // f_e, f_{e+1}, f_{e+2}
  int32_t nbr;     // face beyond this edge << 2 | its local edge, -1 at the boundary
  int32_t flags;   // pseudo-source bits: 1 = a, 2 = b, 4 = c
  int32_t pad[3];
};
static_assert(sizeof(FaceEdge) == 64, "face-edge record");

struct Mesh {
  const FaceEdge* fe;     // [nf][3]
  const int32_t* vf_off;  // [nv + 1]
  const int32_t* vf;      // incident faces: face << 2 | the vertex's corner
};

// A queued item: a window (tag = face << 2 | edge) or a pseudo-source
// (tag = -1 - v, key = its distance).
struct Item {
  double key;
  int32_t tag;
  double b0, b1, sx, sy, sig;
};

// The radius a window's FP32 key is compared with.
__host__ __device__ inline float max_key(double max_dist) {
  return static_cast<float>(max_dist * (1.0 + 1.0 / 65536.0));
}

// The window geometry, shared by both kernels.  St supplies the queue and
// the table of reached vertices: push(Item), dist(v), reach(v, d).
//
// GB300's FP64 rate is about 1/64 of its FP32 rate, so the FP64 work per
// window is kept small: the smallest distance of a window (which only orders
// the queue and bounds the radius) is taken in FP32 and compared with the
// radius widened by 2^-16; the end-vertex filter compares squares instead of
// taking square roots; an edge's unit vector uses the stored 1 / length.
// Distances to vertices stay FP64.  (Divisions through one FP64 Newton step
// from the FP32 reciprocal measured no faster.)
template <class St>
struct Geometry {
  const Mesh& m;
  St& st;
  double max_dist;
  float max_key;  // max_dist widened by 2^-16 (a window's FP32 key errs by ~1e-7)

  // a window on the edge of record E (local edge e of face f), entering f
  __device__ void window(int32_t f, int32_t e, const FaceEdge& E, double b0, double b1, double sx, double sy,
                         double sig) {
    const double L = E.len;
    b0 = fmax(b0, 0.0);
    b1 = fmin(b1, L);
    if (!(b1 - b0 > 1e-12 * L)) return;
    const double x = sx < b0 ? b0 - sx : (sx > b1 ? sx - b1 : 0.0);
    const float key = static_cast<float>(sig) + sqrtf(static_cast<float>(x * x + sy * sy));
    if (key > max_key) return;
    // end-vertex filter, squared: sig + |s - (b1, 0)| > d(P) + b1, and the
    // same at b0 for Q = E.b at L
    const double rP = st.dist(E.a) + b1 - sig;
    const double rQ = st.dist(E.b) + (L - b0) - sig;
    const double fx = sx - b1, nx0 = sx - b0, sy2 = sy * sy;
    if (rP < 0.0 || fx * fx + sy2 > rP * rP) return;
    if (rQ < 0.0 || nx0 * nx0 + sy2 > rQ * rQ) return;
    st.push(Item{static_cast<double>(key), (f << 2) | e, b0, b1, sx, sy, sig});
  }

  // the child crossing face f over its edge of record X (from 2-D point pa,
  // X.a, to pb), covering [q0, q1]; pthird is f's third vertex, on the far
  // side of the edge from the face beyond it
  __device__ void child(const FaceEdge& X, double2 pa, double2 pb, double2 pthird, double2 q0, double2 q1,
                        double sx, double sy, double sig) {
    if (X.nbr < 0) return;
    const int32_t g = X.nbr >> 2, ge = X.nbr & 3;
    const FaceEdge G = m.fe[3 * g + ge];
    const bool same = (G.a == X.a);
    const double2 P = same ? pa : pb, Q = same ? pb : pa;
    const double ux = (Q.x - P.x) * G.inv_len, uy = (Q.y - P.y) * G.inv_len;
    double nx = -uy, ny = ux;
    if (nx * (pthird.x - P.x) + ny * (pthird.y - P.y) > 0.0) {
      nx = -nx;
      ny = -ny;
    }
    const double s2x = (sx - P.x) * ux + (sy - P.y) * uy;
    const double s2y = (sx - P.x) * nx + (sy - P.y) * ny;
    if (!(s2y < 0.0)) return;  // the image lies on the edge's line
    double t0 = (q0.x - P.x) * ux + (q0.y - P.y) * uy;
    double t1 = (q1.x - P.x) * ux + (q1.y - P.y) * uy;
    if (t0 > t1) {
      const double x = t0;
      t0 = t1;
      t1 = x;
    }
    window(g, ge, G, t0, t1, s2x, s2y, sig);
  }

  // where the line from s through (x, 0) meets segment a -> b (clamped)
  __device__ static double2 hit(double sx, double sy, double x, double2 a, double2 b) {
    const double dx = x - sx, dy = -sy;
    const double ex = b.x - a.x, ey = b.y - a.y;
    const double mu = ((sx - a.x) * dy - (sy - a.y) * dx) / (ex * dy - ey * dx);
    const double c = fmin(fmax(mu, 0.0), 1.0);
    return make_double2(a.x + c * ex, a.y + c * ey);
  }

  __device__ void propagate(const Item& w) {
    const int32_t f = w.tag >> 2, e = w.tag & 3;
    // the face's three edge records, loaded together
    const FaceEdge E = m.fe[3 * f + e];
    const FaceEdge Eb = m.fe[3 * f + (e + 1) % 3];  // B -> C
    const FaceEdge Ea = m.fe[3 * f + (e + 2) % 3];  // C -> A
    const double L = E.len;
    const double2 C = make_double2(E.cx, E.cy);
    const double2 A = make_double2(0.0, 0.0), B = make_double2(L, 0.0);
    const double sx = w.sx, sy = w.sy;
    const double xc = sx + (C.x - sx) * (-sy) / (C.y - sy);  // line s -> C at y = 0
    if (xc >= w.b0 && xc <= w.b1) {
      const double dx = C.x - sx, dy = C.y - sy;
      st.reach(E.c, w.sig + sqrt(dx * dx + dy * dy), (E.flags & 4) != 0);
    }
    if (w.b0 < xc) {  // edge C -> A: local edge e + 2
      const double2 q0 = hit(sx, sy, w.b0, A, C);
      const double2 q1 = (w.b1 < xc) ? hit(sx, sy, w.b1, A, C) : C;
      child(Ea, C, A, B, q0, q1, sx, sy, w.sig);
    }
    if (w.b1 > xc) {  // edge B -> C: local edge e + 1
      const double2 q0 = (w.b0 > xc) ? hit(sx, sy, w.b0, B, C) : C;
      const double2 q1 = hit(sx, sy, w.b1, B, C);
      child(Eb, B, C, A, q0, q1, sx, sy, w.sig);
    }
  }

  // a (pseudo-)source u at distance du: its neighbours along the edges, and a
  // window on the edge opposite u in every face around it, entering the face
  // beyond that edge
  __device__ void expand(int32_t u, double du) {
    for (int32_t k = m.vf_off[u]; k < m.vf_off[u + 1]; ++k) {
      const int32_t f = m.vf[k] >> 2, c = m.vf[k] & 3;
      const FaceEdge U1 = m.fe[3 * f + c];            // u -> v1
      const FaceEdge O = m.fe[3 * f + (c + 1) % 3];   // opposite edge v1 -> v2
      const FaceEdge U2 = m.fe[3 * f + (c + 2) % 3];  // v2 -> u
      const double l1 = U1.len, l2 = U2.len;
      st.reach(O.a, du + l1, (O.flags & 1) != 0);
      st.reach(O.b, du + l2, (O.flags & 2) != 0);
      if (O.nbr < 0) continue;
      const int32_t g = O.nbr >> 2, ge = O.nbr & 3;
      const FaceEdge G = m.fe[3 * g + ge];
      const double L = O.len;
      const bool p_is_v1 = (G.a == O.a);
      const double dP = p_is_v1 ? l1 : l2, dQ = p_is_v1 ? l2 : l1;
      const double x = (L * L + dP * dP - dQ * dQ) * (0.5 * O.inv_len);
      const double y2 = dP * dP - x * x;
      const double y = -(y2 > 0.0 ? sqrt(y2) : 0.0);
      if (y < 0.0) window(g, ge, G, 0.0, L, x, y, du);
    }
  }
};

// ---------------------------------------------------------------------------
// One thread per source: a binary heap and an open-addressing table of reached
// vertices in global scratch, element k of thread t at k * T + t.  Used for
// the sources whose propagation outgrows a warp's shared-memory queue.
// ---------------------------------------------------------------------------
struct Scratch {
  double* hkey;   // heap: smallest distance of the item
  int32_t* htag;
  double* hb0;
  double* hb1;
  double* hsx;
  double* hsy;
  double* hsig;
  int32_t* tv;      // table: vertex id, -1 empty
  double* td;       // distance
  double* tdone;    // distance the vertex was expanded at as a pseudo-source
  int32_t* occ;     // occupied table slots, in insertion order
  int32_t hcap;     // heap capacity per thread
  int32_t tbits;    // table capacity per thread = 1 << tbits
};

struct ThreadState {
  const Mesh& m;
  const Scratch& s;
  int64_t t, T;
  int32_t nh = 0, nocc = 0;
  bool fail = false;
  double max_dist;
  __device__ ThreadState(const Mesh& m_, const Scratch& s_, int64_t t_, int64_t T_, double md)
      : m(m_), s(s_), t(t_), T(T_), max_dist(md) {}
  __device__ int64_t ix(int32_t k) const { return static_cast<int64_t>(k) * T + t; }

  __device__ void store(int32_t k, const Item& it) const {
    const int64_t i = ix(k);
    s.hkey[i] = it.key;
    s.htag[i] = it.tag;
    s.hb0[i] = it.b0;
    s.hb1[i] = it.b1;
    s.hsx[i] = it.sx;
    s.hsy[i] = it.sy;
    s.hsig[i] = it.sig;
  }
  __device__ Item load(int32_t k) const {
    const int64_t i = ix(k);
    return Item{s.hkey[i], s.htag[i], s.hb0[i], s.hb1[i], s.hsx[i], s.hsy[i], s.hsig[i]};
  }
  __device__ void push(const Item& it) {
    if (nh >= s.hcap) {
      fail = true;
      return;
    }
    int32_t i = nh++;
    while (i > 0) {
      const int32_t up = (i - 1) >> 1;
      if (s.hkey[ix(up)] <= it.key) break;
      store(i, load(up));
      i = up;
    }
    store(i, it);
  }
  __device__ Item pop() {
    const Item top = load(0);
    const Item last = load(--nh);
    int32_t i = 0;
    for (;;) {
      int32_t c = 2 * i + 1;
      if (c >= nh) break;
      if (c + 1 < nh && s.hkey[ix(c + 1)] < s.hkey[ix(c)]) ++c;
      if (s.hkey[ix(c)] >= last.key) break;
      store(i, load(c));
      i = c;
    }
    if (nh > 0) store(i, last);
    return top;
  }

  // slot of vertex v in the distance table (inserted at +inf when absent and
  // insert is set), or -1
  __device__ int32_t slot(int32_t v, bool insert) {
    const uint32_t mask = (1u << s.tbits) - 1u;
    const uint32_t h = (static_cast<uint32_t>(v) * 2654435761u) >> (32 - s.tbits);
    for (uint32_t p = 0; p <= mask; ++p) {
      const int32_t k = static_cast<int32_t>((h + p) & mask);
      const int32_t key = s.tv[ix(k)];
      if (key == v) return k;
      if (key < 0) {
        if (!insert) return -1;
        if (nocc >= static_cast<int32_t>(3u * (mask + 1u) / 4u)) {
          fail = true;
          return -1;
        }
        s.tv[ix(k)] = v;
        s.td[ix(k)] = INFINITY;
        s.tdone[ix(k)] = INFINITY;
        s.occ[ix(nocc++)] = k;
        return k;
      }
    }
    fail = true;
    return -1;
  }
  __device__ double dist(int32_t v) {
    const int32_t k = slot(v, false);
    return k < 0 ? static_cast<double>(INFINITY) : s.td[ix(k)];
  }
  // d(v) = min(d(v), dv); a pseudo-source whose distance fell is queued
  __device__ void reach(int32_t v, double dv, bool pseudo) {
    const int32_t k = slot(v, true);
    if (k < 0 || !(dv < s.td[ix(k)])) return;
    s.td[ix(k)] = dv;
    if (pseudo && dv <= max_dist) push(Item{dv, -1 - v, 0.0, 0.0, 0.0, 0.0, dv});
  }

  __device__ void run(int32_t src) {
    for (int32_t k = 0; k < nocc; ++k) s.tv[ix(s.occ[ix(k)])] = -1;
    nocc = 0;
    nh = 0;
    fail = false;
    Geometry<ThreadState> geo{m, *this, max_dist, max_key(max_dist)};
    const int32_t k0 = slot(src, true);
    if (k0 < 0) return;
    s.td[ix(k0)] = 0.0;
    s.tdone[ix(k0)] = 0.0;
    geo.expand(src, 0.0);
    for (int64_t it = 0; nh > 0 && !fail; ++it) {
      if (it >= kIterLimit) {
        fail = true;
        return;
      }
      const Item w = pop();
      if (w.key > max_key(max_dist)) break;
      if (w.tag < 0) {
        const int32_t v = -1 - w.tag;
        const int32_t k = slot(v, false);
        if (k < 0 || w.key > s.td[ix(k)] || s.tdone[ix(k)] <= w.key) continue;  // stale or done
        s.tdone[ix(k)] = w.key;
        geo.expand(v, w.key);
      } else {
        geo.propagate(w);
      }
    }
  }
};

// ---------------------------------------------------------------------------
// One warp per source.  The keys of the pending items and the table of
// reached vertices live in the warp's shared memory, the item bodies in
// global memory (per warp, contiguous).  Each round the warp takes up to 32
// items whose key lies within delta of the smallest pending key (one per
// lane), moves the last items into their places, and the lanes propagate
// them together, pushing children and reaching vertices with shared-memory
// atomics.  The filters are sound in any order, so the distances are the
// same exact ones; delta trades a little extra work for 32-wide rounds.
// ---------------------------------------------------------------------------
constexpr int kWarpPool = 2048;            // pending items per warp
constexpr int kWarpTabBits = 10;           // reached-vertex table: 1024 slots
constexpr int kWarpTab = 1 << kWarpTabBits;
constexpr int kWarpTabMax = 3 * kWarpTab / 4;
constexpr int kWarpsPerCta = 6;

struct WarpShared {
  float key[kWarpPool];  // smallest distance of the item, rounded down (orders and bounds only)
  unsigned long long td[kWarpTab];     // distance bits (non-negative doubles order as their bits)
  unsigned long long tdone[kWarpTab];  // distance a pseudo-source was expanded at
  int32_t tv[kWarpTab];                // vertex id, -1 empty
  int32_t occ[kWarpTab];               // occupied slots
  int32_t sel[32];
  int32_t srcpos[32];
  int32_t n_pool;
  int32_t n_occ;
  int32_t fail;
};

struct WarpBodies {  // per warp [kWarpPool]
  int32_t* tag;
  double* b0;
  double* b1;
  double* sx;
  double* sy;
  double* sig;
};

struct WarpState {
  const Mesh& m;
  WarpShared& w;
  WarpBodies b;
  double max_dist;

  __device__ void push(const Item& it) {
    const int32_t i = atomicAdd(&w.n_pool, 1);
    if (i >= kWarpPool) {
      w.fail = 1;
      return;
    }
    w.key[i] = __double2float_rd(it.key);
    b.tag[i] = it.tag;
    b.b0[i] = it.b0;
    b.b1[i] = it.b1;
    b.sx[i] = it.sx;
    b.sy[i] = it.sy;
    b.sig[i] = it.sig;
  }
  // slot of v (claimed with a CAS when absent and insert is set), or -1
  __device__ int32_t slot(int32_t v, bool insert) {
    const uint32_t h = (static_cast<uint32_t>(v) * 2654435761u) >> (32 - kWarpTabBits);
    volatile int32_t* tv = w.tv;
    for (uint32_t p = 0; p < kWarpTab; ++p) {
      const int32_t k = static_cast<int32_t>((h + p) & (kWarpTab - 1));
      int32_t key = tv[k];
      if (key == v) return k;
      if (key < 0) {
        if (!insert) return -1;
        key = atomicCAS(&w.tv[k], -1, v);
        if (key == -1) {
          const int32_t n = atomicAdd(&w.n_occ, 1);
          w.occ[n] = k;  // n < kWarpTab: every claim is one slot
          if (n >= kWarpTabMax) w.fail = 1;
          return k;
        }
        if (key == v) return k;
      }
    }
    w.fail = 1;
    return -1;
  }
  __device__ double dist(int32_t v) {
    const int32_t k = slot(v, false);
    if (k < 0) return static_cast<double>(INFINITY);
    return __longlong_as_double(static_cast<long long>(reinterpret_cast<volatile unsigned long long*>(w.td)[k]));
  }
  __device__ void reach(int32_t v, double dv, bool pseudo) {
    const int32_t k = slot(v, true);
    if (k < 0) return;
    const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(dv));
    const unsigned long long old = atomicMin(&w.td[k], bits);
    if (bits < old && pseudo && dv <= max_dist) push(Item{dv, -1 - v, 0.0, 0.0, 0.0, 0.0, dv});
  }
};

struct LaunchArgs {
  Mesh m;
  Scratch s;                 // thread-per-source kernel
  WarpBodies wb;             // warp kernel: bodies of warp gw at gw * kWarpPool
  const int32_t* src_list;   // sources (nullable: src_lo + q)
  int32_t src_lo;
  int32_t n_src;
  double threshold;
  double max_dist;
  double delta;              // warp kernel: window of keys taken per round
  int32_t only_greater;
  int64_t cap;               // output entries
  int32_t* out_j;
  double* out_d;
  unsigned long long* cursor;
  int32_t* queue;            // warp kernel: next source
  int64_t* src_base;         // [n_src] first output entry of each source (-1: failed)
  int32_t* src_count;        // [n_src]
  int32_t* failed;           // [n_src] sources to run again with more capacity
  int32_t* n_failed;
};

__device__ inline bool keep_pair(const LaunchArgs& a, int32_t src, int32_t v, double d) {
  return v != src && (!a.only_greater || v > src) && d < a.threshold;
}

__global__ void __launch_bounds__(kThreads) geodesic_lists_kernel(LaunchArgs a) {
  const int64_t T = static_cast<int64_t>(gridDim.x) * blockDim.x;
  const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  ThreadState c(a.m, a.s, t, T, a.max_dist);
  for (int64_t q = t; q < a.n_src; q += T) {
    const int32_t src = a.src_list ? a.src_list[q] : a.src_lo + static_cast<int32_t>(q);
    c.run(src);
    if (c.fail) {
      a.src_base[q] = -1;
      a.src_count[q] = 0;
      a.failed[atomicAdd(a.n_failed, 1)] = src;
      continue;
    }
    int32_t n = 0;
    for (int32_t k = 0; k < c.nocc; ++k) {
      const int64_t i = c.ix(a.s.occ[c.ix(k)]);
      n += keep_pair(a, src, a.s.tv[i], a.s.td[i]);
    }
    const unsigned long long base = atomicAdd(a.cursor, static_cast<unsigned long long>(n));
    a.src_base[q] = static_cast<int64_t>(base);
    a.src_count[q] = n;
    int64_t w = static_cast<int64_t>(base);
    for (int32_t k = 0; k < c.nocc; ++k) {
      const int64_t i = c.ix(a.s.occ[c.ix(k)]);
      if (!keep_pair(a, src, a.s.tv[i], a.s.td[i])) continue;
      if (w < a.cap) {
        a.out_j[w] = a.s.tv[i];
        a.out_d[w] = a.s.td[i];
      }
      ++w;
    }
  }
}

__device__ inline double warp_min(double x) {
  for (int o = 16; o > 0; o >>= 1) x = fmin(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}

__global__ void __launch_bounds__(32 * kWarpsPerCta) geodesic_warp_kernel(LaunchArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  WarpShared& w = reinterpret_cast<WarpShared*>(smem_raw)[wid];
  const int64_t gw = static_cast<int64_t>(blockIdx.x) * kWarpsPerCta + wid;
  WarpBodies b = a.wb;
  b.tag += gw * kWarpPool;
  b.b0 += gw * kWarpPool;
  b.b1 += gw * kWarpPool;
  b.sx += gw * kWarpPool;
  b.sy += gw * kWarpPool;
  b.sig += gw * kWarpPool;
  WarpState st{a.m, w, b, a.max_dist};
  Geometry<WarpState> geo{a.m, st, a.max_dist, max_key(a.max_dist)};
  const unsigned all = 0xffffffffu;
  const unsigned lt = (1u << lane) - 1u;
  for (int k = lane; k < kWarpTab; k += 32) {
    w.tv[k] = -1;
    w.td[k] = static_cast<unsigned long long>(__double_as_longlong(static_cast<double>(INFINITY)));
    w.tdone[k] = w.td[k];
  }
  if (lane == 0) w.n_occ = 0;
  __syncwarp();
  for (;;) {
    int32_t q = 0;
    if (lane == 0) q = atomicAdd(a.queue, 1);
    q = __shfl_sync(all, q, 0);
    if (q >= a.n_src) break;
    const int32_t src = a.src_list ? a.src_list[q] : a.src_lo + q;
    // clear the previous source's slots
    const int32_t nocc = w.n_occ;
    __syncwarp();
    for (int32_t k = lane; k < nocc; k += 32) {
      const int32_t s = w.occ[k];
      w.tv[s] = -1;
      w.td[s] = static_cast<unsigned long long>(__double_as_longlong(static_cast<double>(INFINITY)));
      w.tdone[s] = w.td[s];
    }
    if (lane == 0) {
      w.n_occ = 0;
      w.n_pool = 0;
      w.fail = 0;
    }
    __syncwarp();
    if (lane == 0) {
      const int32_t k0 = st.slot(src, true);
      if (k0 >= 0) {
        w.td[k0] = 0ull;
        w.tdone[k0] = 0ull;
        geo.expand(src, 0.0);
      }
    }
    __syncwarp();
    const volatile WarpShared& vw = w;
    for (int64_t round = 0;; ++round) {
      const int32_t n = vw.n_pool;
      if (vw.fail || round >= kIterLimit) {
        if (lane == 0) w.fail = 1;
        break;
      }
      double kmin = static_cast<double>(INFINITY);
      for (int32_t k = lane; k < n; k += 32) kmin = fmin(kmin, static_cast<double>(w.key[k]));
      kmin = warp_min(kmin);
      if (n == 0 || kmin > static_cast<double>(geo.max_key)) break;  // nothing left within the radius
      const double thr = kmin + a.delta;
      // take up to 32 items with key <= thr, in pool order
      int32_t taken = 0;
      for (int32_t base = 0; base < n && taken < 32; base += 32) {
        const int32_t idx = base + lane;
        const bool qual = idx < n && static_cast<double>(w.key[idx]) <= thr;
        const unsigned mk = __ballot_sync(all, qual);
        const int r = __popc(mk & lt);
        if (qual && taken + r < 32) w.sel[taken + r] = idx;
        taken = min(32, taken + __popc(mk));
      }
      __syncwarp();
      Item it{};
      const int32_t my = (lane < taken) ? w.sel[lane] : -1;
      if (my >= 0) it = Item{0.0, b.tag[my], b.b0[my], b.b1[my], b.sx[my], b.sy[my], b.sig[my]};
      __syncwarp();
      if (my >= 0) w.key[my] = -1.0f;  // taken
      __syncwarp();
      // the items beyond the new end that were not taken move into the holes below it
      const int32_t n_new = n - taken;
      const int32_t pos = n_new + lane;
      const bool is_src = lane < taken && w.key[pos] >= 0.0f;
      const unsigned ms = __ballot_sync(all, is_src);
      if (is_src) w.srcpos[__popc(ms & lt)] = pos;
      const bool is_hole = my >= 0 && my < n_new;
      const unsigned mh = __ballot_sync(all, is_hole);
      __syncwarp();
      if (is_hole) {
        const int32_t from = w.srcpos[__popc(mh & lt)];
        w.key[my] = w.key[from];
        b.tag[my] = b.tag[from];
        b.b0[my] = b.b0[from];
        b.b1[my] = b.b1[from];
        b.sx[my] = b.sx[from];
        b.sy[my] = b.sy[from];
        b.sig[my] = b.sig[from];
      }
      __syncwarp();
      if (lane == 0) w.n_pool = n_new;
      __syncwarp();
      if (my >= 0) {
        if (it.tag < 0) {  // a pseudo-source: its exact distance is in sig
          const int32_t v = -1 - it.tag;
          const int32_t k = st.slot(v, false);
          const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(it.sig));
          if (k >= 0 && bits <= reinterpret_cast<volatile unsigned long long*>(w.td)[k] &&
              atomicMin(&w.tdone[k], bits) > bits)
            geo.expand(v, it.sig);
        } else {
          geo.propagate(it);
        }
      }
      __syncwarp();
    }
    __syncwarp();
    if (vw.fail) {
      if (lane == 0) {
        a.src_base[q] = -1;
        a.src_count[q] = 0;
        a.failed[atomicAdd(a.n_failed, 1)] = src;
      }
      __syncwarp();
      continue;
    }
    // output: the reached vertices below the threshold
    const int32_t no = min(w.n_occ, kWarpTab);
    int32_t cnt = 0;
    for (int32_t k = lane; k < no; k += 32) {
      const int32_t s = w.occ[k];
      cnt += keep_pair(a, src, w.tv[s], __longlong_as_double(static_cast<long long>(w.td[s])));
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(all, cnt, o);
    unsigned long long base = 0;
    if (lane == 0) {
      base = atomicAdd(a.cursor, static_cast<unsigned long long>(cnt));
      a.src_base[q] = static_cast<int64_t>(base);
      a.src_count[q] = cnt;
    }
    base = __shfl_sync(all, base, 0);
    int64_t wpos = static_cast<int64_t>(base);
    for (int32_t k0 = 0; k0 < no; k0 += 32) {
      const int32_t k = k0 + lane;
      bool keep = false;
      int32_t v = -1;
      double d = 0.0;
      if (k < no) {
        const int32_t s = w.occ[k];
        v = w.tv[s];
        d = __longlong_as_double(static_cast<long long>(w.td[s]));
        keep = keep_pair(a, src, v, d);
      }
      const unsigned mk = __ballot_sync(all, keep);
      if (keep) {
        const int64_t o = wpos + __popc(mk & lt);
        if (o < a.cap) {
          a.out_j[o] = v;
          a.out_d[o] = d;
        }
      }
      wpos += __popc(mk);
    }
    __syncwarp();
  }
}

}  // namespace geo
}  // namespace tfgb

struct geodesic_mesh {
  int device = 0;
  int32_t nv = 0, nf = 0;
  tfgb::geo::FaceEdge* d_fe = nullptr;
  int32_t* d_vf_off = nullptr;
  int32_t* d_vf = nullptr;
  double pairs_per_src = 256.0;  // output entries per source seen so far (sizes the output buffers)
  int32_t n_saddle = 0;
  double mean_edge = 0.0;
  // results of the last geodesic_distance_lists call, sorted by (i, j)
  std::vector<int32_t> ri, rj;
  std::vector<double> rd;
  std::mutex mu;
};

namespace {

void free_mesh(geodesic_mesh* m) {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaSetDevice(m->device);
  cudaFree(m->d_fe);
  cudaFree(m->d_vf_off);
  cudaFree(m->d_vf);
  cudaSetDevice(dev);
}

struct Buf {
  void* p = nullptr;
  ~Buf() { cudaFree(p); }
};

template <class T>
int upload(T** dst, const std::vector<T>& src) {
  TFGB_CUDA(cudaMalloc(reinterpret_cast<void**>(dst), sizeof(T) * std::max<size_t>(src.size(), 1)));
  if (!src.empty()) TFGB_CUDA(cudaMemcpy(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice));
  return TFCE_OK;
}

// One launch over n_src sources (src_list on the device, or src_lo + q) with
// the given per-thread capacities; appends the output of every source that
// finished and returns the ones that did not in `again`.
// One launch over n_src sources (src_list on the device, or src_lo + q):
// warp mode (hcap == 0) runs one warp per source with its queue keys and
// vertex table in shared memory; otherwise one thread per source with the
// given heap and table capacities in global scratch.  Appends the output of
// every source that finished and returns the ones that did not in `again`.
int launch_chunk(geodesic_mesh* m, const int32_t* h_src, int32_t src_lo, int32_t n_src, double threshold,
                 int32_t only_greater, int32_t hcap, int32_t tbits, double delta, std::vector<int32_t>& out_i,
                 std::vector<int32_t>& out_j, std::vector<double>& out_d, std::vector<int32_t>& again) {
  int sms = 0;
  TFGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->device));
  const bool warp_mode = (hcap == 0);
  const int64_t tcap = warp_mode ? 0 : int64_t(1) << tbits;
  const int64_t per_thread = hcap * (8 + 4 + 5 * 8) + tcap * (4 + 8 + 8 + 4);
  const int64_t budget = int64_t(3) << 30;  // scratch bytes
  constexpr int64_t kB = tfgb::geo::kThreads;
  int64_t T = kB;
  int warp_ctas = 0;
  const size_t warp_smem = sizeof(tfgb::geo::WarpShared) * tfgb::geo::kWarpsPerCta;
  if (warp_mode) {
    TFGB_CUDA(cudaFuncSetAttribute(tfgb::geo::geodesic_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(warp_smem)));
    int per_sm = 0;
    TFGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tfgb::geo::geodesic_warp_kernel,
                                                            32 * tfgb::geo::kWarpsPerCta, warp_smem));
    warp_ctas = sms * std::max(per_sm, 1);
  } else {
    T = std::min<int64_t>(static_cast<int64_t>(sms) * 256, budget / per_thread) / kB * kB;
    T = std::min<int64_t>(std::max<int64_t>(T, kB), (n_src + kB - 1) / kB * kB);
  }
  Buf scratch, srcs, base, count, failed, ctrl, oj, od;
  const int64_t n_warps = static_cast<int64_t>(warp_ctas) * tfgb::geo::kWarpsPerCta;
  const int64_t scratch_bytes = warp_mode ? n_warps * tfgb::geo::kWarpPool * (4 + 5 * 8) : per_thread * T;
  TFGB_CUDA(cudaMalloc(&scratch.p, scratch_bytes + 16 * 256));  // + the 256-byte alignment of the arrays
  char* sp = static_cast<char*>(scratch.p);
  tfgb::geo::Scratch s{};
  tfgb::geo::WarpBodies wb{};
  auto take = [&](int64_t bytes) {
    char* p = sp;
    sp += (bytes + 255) / 256 * 256;
    return p;
  };
  if (warp_mode) {
    const int64_t nb = n_warps * tfgb::geo::kWarpPool;
    wb.b0 = reinterpret_cast<double*>(take(8 * nb));
    wb.b1 = reinterpret_cast<double*>(take(8 * nb));
    wb.sx = reinterpret_cast<double*>(take(8 * nb));
    wb.sy = reinterpret_cast<double*>(take(8 * nb));
    wb.sig = reinterpret_cast<double*>(take(8 * nb));
    wb.tag = reinterpret_cast<int32_t*>(take(4 * nb));
  }
  s.hcap = hcap;
  s.tbits = tbits;
  if (!warp_mode) {
  s.hkey = reinterpret_cast<double*>(take(8 * hcap * T));
  s.hb0 = reinterpret_cast<double*>(take(8 * hcap * T));
  s.hb1 = reinterpret_cast<double*>(take(8 * hcap * T));
  s.hsx = reinterpret_cast<double*>(take(8 * hcap * T));
  s.hsy = reinterpret_cast<double*>(take(8 * hcap * T));
  s.hsig = reinterpret_cast<double*>(take(8 * hcap * T));
  s.td = reinterpret_cast<double*>(take(8 * tcap * T));
  s.tdone = reinterpret_cast<double*>(take(8 * tcap * T));
  s.htag = reinterpret_cast<int32_t*>(take(4 * hcap * T));
  s.tv = reinterpret_cast<int32_t*>(take(4 * tcap * T));
  s.occ = reinterpret_cast<int32_t*>(take(4 * tcap * T));
  }
  if (h_src) {
    TFGB_CUDA(cudaMalloc(&srcs.p, 4 * std::max(n_src, 1)));
    TFGB_CUDA(cudaMemcpy(srcs.p, h_src, 4 * static_cast<size_t>(n_src), cudaMemcpyHostToDevice));
  }
  TFGB_CUDA(cudaMalloc(&base.p, 8 * std::max(n_src, 1)));
  TFGB_CUDA(cudaMalloc(&count.p, 4 * std::max(n_src, 1)));
  TFGB_CUDA(cudaMalloc(&failed.p, 4 * std::max(n_src, 1)));
  TFGB_CUDA(cudaMalloc(&ctrl.p, 16));  // cursor (8 bytes), failed count, warp queue
  // output entries, from the largest count per source seen on this mesh; a
  // launch that outgrows it runs again with the exact size
  int64_t cap = std::max<int64_t>(static_cast<int64_t>(n_src * m->pairs_per_src * 1.25), 4096);
  for (int attempt = 0; attempt < 2; ++attempt) {
    cudaFree(oj.p);
    cudaFree(od.p);
    oj.p = od.p = nullptr;
    TFGB_CUDA(cudaMalloc(&oj.p, 4 * cap));
    TFGB_CUDA(cudaMalloc(&od.p, 8 * cap));
    TFGB_CUDA(cudaMemset(ctrl.p, 0, 16));
    // every table slot empty (-1): a thread clears only the slots its own
    // sources filled, so a relaunch starts from a cleared table too (the
    // warp kernel clears its shared-memory table itself)
    if (!warp_mode) TFGB_CUDA(cudaMemset(s.tv, 0xff, 4 * tcap * T));
    tfgb::geo::LaunchArgs a{};
    a.m.fe = m->d_fe;
    a.m.vf_off = m->d_vf_off;
    a.m.vf = m->d_vf;
    a.s = s;
    a.wb = wb;
    a.delta = delta;
    a.queue = reinterpret_cast<int32_t*>(static_cast<char*>(ctrl.p) + 12);
    a.src_list = static_cast<const int32_t*>(srcs.p);
    a.src_lo = src_lo;
    a.n_src = n_src;
    a.threshold = threshold;
    a.max_dist = threshold + 1e-10;  // adjacency.pyx:54
    a.only_greater = only_greater;
    a.cap = cap;
    a.out_j = static_cast<int32_t*>(oj.p);
    a.out_d = static_cast<double*>(od.p);
    a.cursor = static_cast<unsigned long long*>(ctrl.p);
    a.n_failed = reinterpret_cast<int32_t*>(static_cast<char*>(ctrl.p) + 8);
    a.src_base = static_cast<int64_t*>(base.p);
    a.src_count = static_cast<int32_t*>(count.p);
    a.failed = static_cast<int32_t*>(failed.p);
    if (warp_mode)
      tfgb::geo::geodesic_warp_kernel<<<warp_ctas, 32 * tfgb::geo::kWarpsPerCta, warp_smem>>>(a);
    else
      tfgb::geo::geodesic_lists_kernel<<<static_cast<unsigned>(T / tfgb::geo::kThreads), tfgb::geo::kThreads>>>(a);
    TFGB_CUDA(cudaGetLastError());
    TFGB_CUDA(cudaDeviceSynchronize());
    unsigned long long used = 0;
    TFGB_CUDA(cudaMemcpy(&used, ctrl.p, 8, cudaMemcpyDeviceToHost));
    m->pairs_per_src = std::max(m->pairs_per_src, static_cast<double>(used) / std::max(n_src, 1));
    if (static_cast<int64_t>(used) <= cap) break;
    cap = static_cast<int64_t>(used);  // run the chunk again with room for all of it
  }
  int32_t n_failed = 0;
  TFGB_CUDA(cudaMemcpy(&n_failed, static_cast<char*>(ctrl.p) + 8, 4, cudaMemcpyDeviceToHost));
  std::vector<int64_t> hb(n_src);
  std::vector<int32_t> hc(n_src);
  unsigned long long used = 0;
  TFGB_CUDA(cudaMemcpy(&used, ctrl.p, 8, cudaMemcpyDeviceToHost));
  std::vector<int32_t> hj(used);
  std::vector<double> hd(used);
  if (n_src) {
    TFGB_CUDA(cudaMemcpy(hb.data(), base.p, 8 * static_cast<size_t>(n_src), cudaMemcpyDeviceToHost));
    TFGB_CUDA(cudaMemcpy(hc.data(), count.p, 4 * static_cast<size_t>(n_src), cudaMemcpyDeviceToHost));
  }
  if (used) {
    TFGB_CUDA(cudaMemcpy(hj.data(), oj.p, 4 * used, cudaMemcpyDeviceToHost));
    TFGB_CUDA(cudaMemcpy(hd.data(), od.p, 8 * used, cudaMemcpyDeviceToHost));
  }
  if (n_failed) {
    const size_t n0 = again.size();
    again.resize(n0 + n_failed);
    TFGB_CUDA(cudaMemcpy(again.data() + n0, failed.p, 4 * static_cast<size_t>(n_failed), cudaMemcpyDeviceToHost));
  }
  // every finished source's block, its entries sorted by j
  std::vector<int32_t> order;
  for (int32_t q = 0; q < n_src; ++q) {
    if (hb[q] < 0) continue;
    const int32_t src = h_src ? h_src[q] : src_lo + q;
    order.resize(hc[q]);
    std::iota(order.begin(), order.end(), 0);
    const int32_t* jj = hj.data() + hb[q];
    std::sort(order.begin(), order.end(), [&](int32_t x, int32_t y) { return jj[x] < jj[y]; });
    for (int32_t k : order) {
      out_i.push_back(src);
      out_j.push_back(jj[k]);
      out_d.push_back(hd[hb[q] + k]);
    }
  }
  return TFCE_OK;
}

double edge_len(const float* p, int32_t a, int32_t b) {
  const double x = (double)p[3 * a] - (double)p[3 * b];
  const double y = (double)p[3 * a + 1] - (double)p[3 * b + 1];
  const double z = (double)p[3 * a + 2] - (double)p[3 * b + 2];
  return std::sqrt(x * x + y * y + z * z);
}

}  // namespace

extern "C" {

int geodesic_mesh_create(const float* pts, int32_t n_vertices, const int32_t* faces, int32_t n_faces,
                         geodesic_mesh** out) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(out != nullptr, "out is NULL");
  *out = nullptr;
  TFGB_CHECK_ARG(pts && faces, "NULL pointer");
  TFGB_CHECK_ARG(n_vertices > 0 && n_faces > 0, "empty mesh");
  TFGB_CHECK_ARG(n_faces <= (INT32_MAX >> 2) / 3, "too many faces");
  const int64_t nf = n_faces, nv = n_vertices;
  for (int64_t k = 0; k < 3 * nf; ++k)
    TFGB_CHECK_ARG(faces[k] >= 0 && faces[k] < n_vertices, "face vertex index out of range");
  for (int64_t k = 0; k < 3 * nv; ++k) TFGB_CHECK_ARG(std::isfinite(pts[k]), "non-finite vertex coordinate");
  std::vector<double> len(3 * nf);
  std::vector<double2> third(3 * nf);
  std::vector<int32_t> nbr(3 * nf, -1);
  std::vector<std::pair<uint64_t, int32_t>> keys(3 * nf);
  for (int64_t f = 0; f < nf; ++f) {
    const int32_t* v = faces + 3 * f;
    TFGB_CHECK_ARG(v[0] != v[1] && v[1] != v[2] && v[2] != v[0], "face with a repeated vertex");
    for (int e = 0; e < 3; ++e) {
      const int32_t a = v[e], b = v[(e + 1) % 3];
      len[3 * f + e] = edge_len(pts, a, b);
      TFGB_CHECK_ARG(len[3 * f + e] > 0.0, "zero-length edge");
      const uint64_t lo = static_cast<uint32_t>(std::min(a, b)), hi = static_cast<uint32_t>(std::max(a, b));
      keys[3 * f + e] = {(lo << 32) | hi, static_cast<int32_t>(3 * f + e)};
    }
    for (int e = 0; e < 3; ++e) {  // the third vertex in the frame of edge e
      const double L = len[3 * f + e], la = len[3 * f + (e + 2) % 3], lb = len[3 * f + (e + 1) % 3];
      const double cx = (L * L + la * la - lb * lb) / (2.0 * L);
      const double cy2 = la * la - cx * cx;
      third[3 * f + e] = make_double2(cx, cy2 > 0.0 ? std::sqrt(cy2) : 0.0);
      TFGB_CHECK_ARG(cy2 > 0.0, "degenerate (zero-area) face");
    }
  }
  std::sort(keys.begin(), keys.end());
  for (size_t k = 0; k + 1 < keys.size(); ++k) {
    if (keys[k].first != keys[k + 1].first) continue;
    TFGB_CHECK_ARG(k + 2 >= keys.size() || keys[k + 2].first != keys[k].first, "edge shared by more than two faces");
    const int32_t s0 = keys[k].second, s1 = keys[k + 1].second;
    nbr[s0] = ((s1 / 3) << 2) | (s1 % 3);
    nbr[s1] = ((s0 / 3) << 2) | (s0 % 3);
    ++k;
  }
  std::vector<int32_t> vf_off(nv + 1, 0), vf(3 * nf);
  std::vector<double> angle(nv, 0.0);
  std::vector<uint8_t> saddle(nv, 0);
  for (int64_t k = 0; k < 3 * nf; ++k) vf_off[faces[k] + 1]++;
  for (int64_t v = 0; v < nv; ++v) vf_off[v + 1] += vf_off[v];
  std::vector<int32_t> fill(vf_off.begin(), vf_off.end() - 1);
  for (int64_t f = 0; f < nf; ++f) {
    for (int c = 0; c < 3; ++c) {
      const int32_t v = faces[3 * f + c];
      vf[fill[v]++] = static_cast<int32_t>((f << 2) | c);
      // corner angle at v (between its two edges in face f)
      const double lo = len[3 * f + (c + 1) % 3], l1 = len[3 * f + c], l2 = len[3 * f + (c + 2) % 3];
      double cs = (l1 * l1 + l2 * l2 - lo * lo) / (2.0 * l1 * l2);
      cs = cs > 1.0 ? 1.0 : (cs < -1.0 ? -1.0 : cs);
      angle[v] += std::acos(cs);
      if (nbr[3 * f + c] < 0) {  // boundary edge: both ends are pseudo-sources
        saddle[faces[3 * f + c]] = 1;
        saddle[faces[3 * f + (c + 1) % 3]] = 1;
      }
    }
  }
  int32_t n_saddle = 0;
  for (int64_t v = 0; v < nv; ++v) {
    if (angle[v] > 6.283185307179586477 - 1e-5) saddle[v] = 1;  // geodesic_mesh.h:335
    n_saddle += saddle[v];
  }
  auto* m = new geodesic_mesh();
  TFGB_CUDA(cudaGetDevice(&m->device));
  m->nv = n_vertices;
  m->nf = n_faces;
  m->n_saddle = n_saddle;
  m->mean_edge = std::accumulate(len.begin(), len.end(), 0.0) / static_cast<double>(len.size());
  std::vector<tfgb::geo::FaceEdge> fe(3 * nf);
  for (int64_t f = 0; f < nf; ++f) {
    for (int e = 0; e < 3; ++e) {
      tfgb::geo::FaceEdge& r = fe[3 * f + e];
      r.len = len[3 * f + e];
      r.inv_len = 1.0 / len[3 * f + e];
      r.cx = third[3 * f + e].x;
      r.cy = third[3 * f + e].y;
      r.a = faces[3 * f + e];
      r.b = faces[3 * f + (e + 1) % 3];
      r.c = faces[3 * f + (e + 2) % 3];
      r.nbr = nbr[3 * f + e];
      r.flags = (saddle[r.a] ? 1 : 0) | (saddle[r.b] ? 2 : 0) | (saddle[r.c] ? 4 : 0);
      r.pad[0] = r.pad[1] = r.pad[2] = 0;
    }
  }
  int rc = upload(&m->d_fe, fe);
  if (!rc) rc = upload(&m->d_vf_off, vf_off);
  if (!rc) rc = upload(&m->d_vf, vf);
  if (rc) {
    free_mesh(m);
    delete m;
    return rc;
  }
  *out = m;
  return TFCE_OK;
}

void geodesic_mesh_destroy(geodesic_mesh* m) {
  if (!m) return;
  free_mesh(m);
  delete m;
}

int geodesic_mesh_saddles(geodesic_mesh* m, int32_t* n_saddle) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(m && n_saddle, "NULL pointer");
  *n_saddle = m->n_saddle;
  return TFCE_OK;
}

int geodesic_distance_lists(geodesic_mesh* m, double threshold, int32_t only_greater, int32_t src_lo,
                            int32_t src_hi, int64_t* n_out) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(m && n_out, "NULL pointer");
  *n_out = 0;
  TFGB_CHECK_ARG(std::isfinite(threshold) && threshold > 0.0, "threshold must be finite and > 0");
  TFGB_CHECK_ARG(0 <= src_lo && src_lo <= src_hi && src_hi <= m->nv, "source range outside the mesh");
  std::lock_guard<std::mutex> lk(m->mu);
  int dev = 0;
  TFGB_CUDA(cudaGetDevice(&dev));
  TFGB_CUDA(cudaSetDevice(m->device));
  std::vector<int32_t> ci, cj, again;
  std::vector<double> cd;
  int rc = TFCE_OK;
  constexpr int32_t kChunk = 1 << 16;
  // keys within delta of the frontier are taken together: one mean edge length
  double delta = m->mean_edge;
  if (const char* env = std::getenv("TFCE_GEODESIC_DELTA_EDGES")) delta = std::atof(env) * m->mean_edge;
  for (int32_t lo = src_lo; lo < src_hi && !rc; lo += kChunk) {
    const int32_t n = std::min(kChunk, src_hi - lo);
    rc = launch_chunk(m, nullptr, lo, n, threshold, only_greater, 0, 0, delta, ci, cj, cd, again);
  }
  // sources that outgrew a warp's queue or table: one thread each, with 4096
  // and then 16384 heap entries and table slots in global scratch
  for (int round = 1; round <= 2 && !rc && !again.empty(); ++round) {
    std::vector<int32_t> todo;
    todo.swap(again);
    rc = launch_chunk(m, todo.data(), 0, static_cast<int32_t>(todo.size()), threshold, only_greater,
                      1024 << (2 * round), 10 + 2 * round, delta, ci, cj, cd, again);
  }
  cudaSetDevice(dev);
  if (rc) return rc;
  if (!again.empty()) {
    tfgb::set_error("geodesic propagation of %zu source(s) outgrew 16384 heap entries / table slots",
                    again.size());
    return TFCE_ERANGE;
  }
  // blocks of one source are contiguous and sorted by j; order them by source
  std::vector<int64_t> start(static_cast<size_t>(src_hi - src_lo) + 1, 0);
  for (int32_t i : ci) start[i - src_lo + 1]++;
  for (size_t k = 1; k < start.size(); ++k) start[k] += start[k - 1];
  m->ri.assign(ci.size(), 0);
  m->rj.assign(ci.size(), 0);
  m->rd.assign(ci.size(), 0.0);
  std::vector<int64_t> pos(start.begin(), start.end() - 1);
  for (size_t k = 0; k < ci.size(); ++k) {
    const int64_t w = pos[ci[k] - src_lo]++;
    m->ri[w] = ci[k];
    m->rj[w] = cj[k];
    m->rd[w] = cd[k];
  }
  *n_out = static_cast<int64_t>(ci.size());
  return TFCE_OK;
}

int geodesic_take_lists(geodesic_mesh* m, int32_t* out_i, int32_t* out_j, double* out_d, int64_t cap) {
  tfgb::clear_error();
  TFGB_CHECK_ARG(m != nullptr, "NULL mesh");
  std::lock_guard<std::mutex> lk(m->mu);
  const int64_t n = static_cast<int64_t>(m->ri.size());
  TFGB_CHECK_ARG(cap >= n, "output capacity below the list length");
  TFGB_CHECK_ARG(n == 0 || (out_i && out_j && out_d), "NULL output");
  if (n) {
    std::memcpy(out_i, m->ri.data(), sizeof(int32_t) * n);
    std::memcpy(out_j, m->rj.data(), sizeof(int32_t) * n);
    std::memcpy(out_d, m->rd.data(), sizeof(double) * n);
  }
  std::vector<int32_t>().swap(m->ri);
  std::vector<int32_t>().swap(m->rj);
  std::vector<double>().swap(m->rd);
  return TFCE_OK;
}

}  // extern "C"

