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
// beyond the radius.  Windows and pseudo-sources are taken in order of their
// smallest distance from a binary heap until it exceeds the radius.
//
// GPU mapping: sources are independent, so each thread runs the propagation
// of one source at a time (a grid-stride loop over the sources).  Its heap
// (windows stored inline) and its open-addressing table of vertex distances
// live in global scratch laid out [slot][thread], so the threads of a warp
// touching the same heap level or table slot coalesce.  The mesh tables are
// read-only and shared by all threads (L2-resident: ~100 bytes per face).
// A source whose heap or table outgrows its capacity is listed and run again
// with four times the capacity; every loop is bounded.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <numeric>
#include <vector>

#include "common.cuh"

namespace tfgb {
namespace geo {

constexpr int kThreads = 128;
constexpr int64_t kIterLimit = int64_t(1) << 22;  // heap pops per source

struct Mesh {
  const int32_t* face;    // [nf][3]
  const int32_t* nbr;     // [nf][3] face beyond local edge e << 2 | its local edge, -1 at the boundary
  const double* len;      // [nf][3] length of local edge e (f_e -> f_{e+1})
  const double2* third;   // [nf][3] third vertex in the frame of local edge e
  const int32_t* vf_off;  // [nv + 1]
  const int32_t* vf;      // incident faces: face << 2 | the vertex's corner
  const uint8_t* saddle;  // [nv]
};

// Per-thread scratch, element k of thread t at k * T + t.
struct Scratch {
  double* hkey;   // heap: smallest distance of the item
  int32_t* htag;  // face << 2 | edge of a window, or -1 - v for a pseudo-source v
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

struct Item {
  double key;
  int32_t tag;
  double b0, b1, sx, sy, sig;
};

struct Ctx {
  const Mesh& m;
  const Scratch& s;
  int64_t t, T;
  int32_t nh = 0, nocc = 0;
  bool fail = false;
  double max_dist;
  __device__ Ctx(const Mesh& m_, const Scratch& s_, int64_t t_, int64_t T_, double md)
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
  __device__ void reach(int32_t v, double dv) {
    const int32_t k = slot(v, true);
    if (k < 0 || !(dv < s.td[ix(k)])) return;
    s.td[ix(k)] = dv;
    if (m.saddle[v] && dv <= max_dist) push(Item{dv, -1 - v, 0.0, 0.0, 0.0, 0.0, 0.0});
  }

  // a window on local edge e of face f, entering f
  __device__ void window(int32_t f, int32_t e, double b0, double b1, double sx, double sy, double sig) {
    const double L = m.len[3 * f + e];
    b0 = fmax(b0, 0.0);
    b1 = fmin(b1, L);
    if (!(b1 - b0 > 1e-12 * L)) return;
    const double x = sx < b0 ? b0 - sx : (sx > b1 ? sx - b1 : 0.0);
    const double key = sig + sqrt(x * x + sy * sy);
    if (key > max_dist) return;
    // end-vertex filter: P = f_e at 0, Q = f_{e+1} at L
    const double dP = dist(m.face[3 * f + e]);
    const double dQ = dist(m.face[3 * f + (e + 1) % 3]);
    const double far = sig + hypot(sx - b1, sy), near = sig + hypot(sx - b0, sy);
    if (far > dP + b1 || near > dQ + (L - b0)) return;
    push(Item{key, (f << 2) | e, b0, b1, sx, sy, sig});
  }

  // the child crossing face f over its local edge le, from 2-D point pa (the
  // edge's first vertex in f) to pb, covering [q0, q1]; pthird is f's third
  // vertex, on the far side of the edge from the face beyond it
  __device__ void child(int32_t f, int32_t le, double2 pa, double2 pb, double2 pthird, double2 q0, double2 q1,
                        double sx, double sy, double sig) {
    const int32_t nb = m.nbr[3 * f + le];
    if (nb < 0) return;
    const int32_t g = nb >> 2, ge = nb & 3;
    const bool same = (m.face[3 * g + ge] == m.face[3 * f + le]);
    const double2 P = same ? pa : pb, Q = same ? pb : pa;
    double ux = Q.x - P.x, uy = Q.y - P.y;
    const double ul = hypot(ux, uy);
    ux /= ul;
    uy /= ul;
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
    window(g, ge, t0, t1, s2x, s2y, sig);
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
    const double L = m.len[3 * f + e];
    const double2 C = m.third[3 * f + e];
    const double2 A = make_double2(0.0, 0.0), B = make_double2(L, 0.0);
    const double sx = w.sx, sy = w.sy;
    const double xc = sx + (C.x - sx) * (-sy) / (C.y - sy);  // line s -> C at y = 0
    if (xc >= w.b0 && xc <= w.b1) reach(m.face[3 * f + (e + 2) % 3], w.sig + hypot(C.x - sx, C.y - sy));
    if (w.b0 < xc) {  // edge C -> A: local edge e + 2
      const double2 q0 = hit(sx, sy, w.b0, A, C);
      const double2 q1 = (w.b1 < xc) ? hit(sx, sy, w.b1, A, C) : C;
      child(f, (e + 2) % 3, C, A, B, q0, q1, sx, sy, w.sig);
    }
    if (w.b1 > xc) {  // edge B -> C: local edge e + 1
      const double2 q0 = (w.b0 > xc) ? hit(sx, sy, w.b0, B, C) : C;
      const double2 q1 = hit(sx, sy, w.b1, B, C);
      child(f, (e + 1) % 3, B, C, A, q0, q1, sx, sy, w.sig);
    }
  }

  // a (pseudo-)source u at distance du: its neighbours along the edges, and a
  // window on the edge opposite u in every face around it, entering the face
  // beyond that edge
  __device__ void expand(int32_t u, double du) {
    for (int32_t k = m.vf_off[u]; k < m.vf_off[u + 1] && !fail; ++k) {
      const int32_t f = m.vf[k] >> 2, c = m.vf[k] & 3;
      const int32_t e = (c + 1) % 3;  // opposite edge f_{c+1} -> f_{c+2}
      const int32_t v1 = m.face[3 * f + e], v2 = m.face[3 * f + (e + 1) % 3];
      const double l1 = m.len[3 * f + c];            // u -> v1
      const double l2 = m.len[3 * f + (c + 2) % 3];  // v2 -> u
      reach(v1, du + l1);
      reach(v2, du + l2);
      const int32_t nb = m.nbr[3 * f + e];
      if (nb < 0) continue;
      const int32_t g = nb >> 2, ge = nb & 3;
      const double L = m.len[3 * f + e];
      const bool p_is_v1 = (m.face[3 * g + ge] == v1);
      const double dP = p_is_v1 ? l1 : l2, dQ = p_is_v1 ? l2 : l1;
      const double x = (L * L + dP * dP - dQ * dQ) / (2.0 * L);
      const double y2 = dP * dP - x * x;
      const double y = -(y2 > 0.0 ? sqrt(y2) : 0.0);
      if (y < 0.0) window(g, ge, 0.0, L, x, y, du);
    }
  }

  __device__ void run(int32_t src) {
    for (int32_t k = 0; k < nocc; ++k) s.tv[ix(s.occ[ix(k)])] = -1;
    nocc = 0;
    nh = 0;
    fail = false;
    const int32_t k0 = slot(src, true);
    if (k0 < 0) return;
    s.td[ix(k0)] = 0.0;
    s.tdone[ix(k0)] = 0.0;
    expand(src, 0.0);
    for (int64_t it = 0; nh > 0 && !fail; ++it) {
      if (it >= kIterLimit) {
        fail = true;
        return;
      }
      const Item w = pop();
      if (w.key > max_dist) break;
      if (w.tag < 0) {
        const int32_t v = -1 - w.tag;
        const int32_t k = slot(v, false);
        if (k < 0 || w.key > s.td[ix(k)] || s.tdone[ix(k)] <= w.key) continue;  // stale or done
        s.tdone[ix(k)] = w.key;
        expand(v, w.key);
      } else {
        propagate(w);
      }
    }
  }
};

struct LaunchArgs {
  Mesh m;
  Scratch s;
  const int32_t* src_list;  // sources (nullable: src_lo + q)
  int32_t src_lo;
  int32_t n_src;
  double threshold;
  double max_dist;
  int32_t only_greater;
  int64_t cap;               // output entries
  int32_t* out_j;
  double* out_d;
  unsigned long long* cursor;
  int64_t* src_base;         // [n_src] first output entry of each source (-1: failed)
  int32_t* src_count;        // [n_src]
  int32_t* failed;           // [n_src] sources to run again with more capacity
  int32_t* n_failed;
};

__global__ void __launch_bounds__(kThreads) geodesic_lists_kernel(LaunchArgs a) {
  const int64_t T = static_cast<int64_t>(gridDim.x) * blockDim.x;
  const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  Ctx c(a.m, a.s, t, T, a.max_dist);
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
      const int32_t v = a.s.tv[i];
      if (v != src && (!a.only_greater || v > src) && a.s.td[i] < a.threshold) ++n;
    }
    const unsigned long long base = atomicAdd(a.cursor, static_cast<unsigned long long>(n));
    a.src_base[q] = static_cast<int64_t>(base);
    a.src_count[q] = n;
    int64_t w = static_cast<int64_t>(base);
    for (int32_t k = 0; k < c.nocc; ++k) {
      const int64_t i = c.ix(a.s.occ[c.ix(k)]);
      const int32_t v = a.s.tv[i];
      const double d = a.s.td[i];
      if (v != src && (!a.only_greater || v > src) && d < a.threshold) {
        if (w < a.cap) {
          a.out_j[w] = v;
          a.out_d[w] = d;
        }
        ++w;
      }
    }
  }
}

}  // namespace geo
}  // namespace tfgb

struct geodesic_mesh {
  int device = 0;
  int32_t nv = 0, nf = 0;
  int32_t* d_face = nullptr;
  int32_t* d_nbr = nullptr;
  double* d_len = nullptr;
  double2* d_third = nullptr;
  int32_t* d_vf_off = nullptr;
  int32_t* d_vf = nullptr;
  uint8_t* d_saddle = nullptr;
  int32_t n_saddle = 0;
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
  cudaFree(m->d_face);
  cudaFree(m->d_nbr);
  cudaFree(m->d_len);
  cudaFree(m->d_third);
  cudaFree(m->d_vf_off);
  cudaFree(m->d_vf);
  cudaFree(m->d_saddle);
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
int launch_chunk(geodesic_mesh* m, const int32_t* h_src, int32_t src_lo, int32_t n_src, double threshold,
                 int32_t only_greater, int32_t hcap, int32_t tbits, std::vector<int32_t>& out_i,
                 std::vector<int32_t>& out_j, std::vector<double>& out_d, std::vector<int32_t>& again) {
  int sms = 0;
  TFGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->device));
  const int64_t tcap = int64_t(1) << tbits;
  const int64_t per_thread = hcap * (8 + 4 + 5 * 8) + tcap * (4 + 8 + 8 + 4);
  const int64_t budget = int64_t(3) << 30;  // scratch bytes
  constexpr int64_t kB = tfgb::geo::kThreads;
  int64_t T = std::min<int64_t>(static_cast<int64_t>(sms) * 256, budget / per_thread) / kB * kB;
  T = std::min<int64_t>(std::max<int64_t>(T, kB), (n_src + kB - 1) / kB * kB);
  Buf scratch, srcs, base, count, failed, ctrl, oj, od;
  TFGB_CUDA(cudaMalloc(&scratch.p, per_thread * T + 16 * 256));  // + the 256-byte alignment of 11 arrays
  char* sp = static_cast<char*>(scratch.p);
  tfgb::geo::Scratch s{};
  auto take = [&](int64_t bytes) {
    char* p = sp;
    sp += (bytes + 255) / 256 * 256;
    return p;
  };
  s.hcap = hcap;
  s.tbits = tbits;
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
  (void)sp;
  if (h_src) {
    TFGB_CUDA(cudaMalloc(&srcs.p, 4 * std::max(n_src, 1)));
    TFGB_CUDA(cudaMemcpy(srcs.p, h_src, 4 * static_cast<size_t>(n_src), cudaMemcpyHostToDevice));
  }
  TFGB_CUDA(cudaMalloc(&base.p, 8 * std::max(n_src, 1)));
  TFGB_CUDA(cudaMalloc(&count.p, 4 * std::max(n_src, 1)));
  TFGB_CUDA(cudaMalloc(&failed.p, 4 * std::max(n_src, 1)));
  TFGB_CUDA(cudaMalloc(&ctrl.p, 16));
  int64_t cap = std::max<int64_t>(int64_t(n_src) * 256, 4096);  // output entries; relaunched larger when short
  for (int attempt = 0; attempt < 2; ++attempt) {
    cudaFree(oj.p);
    cudaFree(od.p);
    oj.p = od.p = nullptr;
    TFGB_CUDA(cudaMalloc(&oj.p, 4 * cap));
    TFGB_CUDA(cudaMalloc(&od.p, 8 * cap));
    TFGB_CUDA(cudaMemset(ctrl.p, 0, 16));
    // every table slot empty (-1): a thread clears only the slots its own
    // sources filled, so a relaunch starts from a cleared table too
    TFGB_CUDA(cudaMemset(s.tv, 0xff, 4 * tcap * T));
    tfgb::geo::LaunchArgs a{};
    a.m.face = m->d_face;
    a.m.nbr = m->d_nbr;
    a.m.len = m->d_len;
    a.m.third = m->d_third;
    a.m.vf_off = m->d_vf_off;
    a.m.vf = m->d_vf;
    a.m.saddle = m->d_saddle;
    a.s = s;
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
    tfgb::geo::geodesic_lists_kernel<<<static_cast<unsigned>(T / tfgb::geo::kThreads), tfgb::geo::kThreads>>>(a);
    TFGB_CUDA(cudaGetLastError());
    TFGB_CUDA(cudaDeviceSynchronize());
    unsigned long long used = 0;
    TFGB_CUDA(cudaMemcpy(&used, ctrl.p, 8, cudaMemcpyDeviceToHost));
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
  int rc = upload(&m->d_face, std::vector<int32_t>(faces, faces + 3 * nf));
  if (!rc) rc = upload(&m->d_nbr, nbr);
  if (!rc) rc = upload(&m->d_len, len);
  if (!rc) rc = upload(&m->d_third, third);
  if (!rc) rc = upload(&m->d_vf_off, vf_off);
  if (!rc) rc = upload(&m->d_vf, vf);
  if (!rc) rc = upload(&m->d_saddle, saddle);
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
  for (int32_t lo = src_lo; lo < src_hi && !rc; lo += kChunk) {
    const int32_t n = std::min(kChunk, src_hi - lo);
    rc = launch_chunk(m, nullptr, lo, n, threshold, only_greater, 1024, 10, ci, cj, cd, again);
  }
  // sources that outgrew the heap or the distance table: four times the room
  for (int round = 1; round <= 2 && !rc && !again.empty(); ++round) {
    std::vector<int32_t> todo;
    todo.swap(again);
    rc = launch_chunk(m, todo.data(), 0, static_cast<int32_t>(todo.size()), threshold, only_greater,
                      1024 << (2 * round), 10 + 2 * round, ci, cj, cd, again);
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

