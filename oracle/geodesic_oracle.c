/* ORACLE -- test infrastructure, not product code.
 *
 * Exact geodesic distances on a triangle mesh from each source vertex to the
 * vertices within a radius: the quantity tfce_mediation/adjacency.pyx:44-106
 * (compute, compute_distance_parallel) obtains from the reference's exact
 * geodesic library (tfce_mediation/lib/geodesic/geodesic_algorithm_exact.h,
 * Kirsanov's implementation of Mitchell-Mount-Papadimitriou).
 *
 * This restatement computes the same exact distances with the window
 * propagation of Chen and Han as improved by Xin and Wang ("Improving Chen
 * and Han's algorithm on the discrete geodesic problem", ACM TOG 28(4), 2009):
 *   - a window is an interval [b0, b1] of a face edge, the unfolded image s of
 *     its (pseudo-)source in the 2-D frame of that edge and the distance sigma
 *     from the source to that image; the distance it gives to a point p of the
 *     interval is sigma + |s - p|;
 *   - a window crosses the face beyond its edge and splits at the face's third
 *     vertex C into at most two children on the other two edges; C is reached
 *     when the line from s to C passes through the interval;
 *   - a vertex whose total angle exceeds 2 pi - 1e-5, or that lies on the mesh
 *     boundary, is a pseudo-source (the reference's rule,
 *     geodesic_mesh.h:335-344): it starts windows on the edges opposite it;
 *   - a window is dropped when one of the edge's end vertices gives a shorter
 *     path to every point of the interval (d(P) + t shorter at the far end or
 *     d(Q) + L - t shorter at the near end: the differences are monotone along
 *     the edge), or when it lies beyond the radius;
 *   - windows and pseudo-sources are processed in order of their smallest
 *     distance (binary heap), stopping once it exceeds the radius.
 * Double precision throughout, from the float32 coordinates the reference
 * takes.  Output: (i, j, d) for every source i in [src_lo, src_hi) and vertex
 * j with d < threshold (only j > i when only_greater, as
 * compute_distance_parallel lists them), sorted by i then j.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define GEO_TWO_PI 6.283185307179586477

typedef struct {
  int32_t nf;        /* faces */
  int32_t nv;        /* vertices */
  const int32_t* f;  /* [nf][3] */
  double* p;         /* [nv][3] */
  int32_t* nbr;      /* [nf][3]: face across local edge e (f_e -> f_{e+1}), -1 at the boundary */
  int32_t* nbr_e;    /* [nf][3]: that edge's local index in the neighbour */
  double* len;       /* [nf][3]: length of local edge e */
  int64_t* vf_off;   /* [nv+1] incident faces of a vertex */
  int32_t* vf;       /* incident face ids */
  uint8_t* saddle;   /* [nv] */
} GMesh;

typedef struct {
  int32_t face, edge;
  double b0, b1, sx, sy, sigma;
} GWin;

typedef struct {
  double key;
  int32_t idx;   /* window index, or vertex id when vert */
  int32_t vert;
} GItem;

typedef struct {
  GWin* w;
  int64_t nw, cw;
  GItem* h;
  int64_t nh, ch;
  double* d;        /* [nv] distance, INFINITY when not reached */
  double* done;     /* [nv] distance a pseudo-source was expanded at */
  int32_t* touched; /* vertices whose d or done was set */
  int64_t nt, ct;
} GState;

static double glen(const double* a, const double* b) {
  const double x = a[0] - b[0], y = a[1] - b[1], z = a[2] - b[2];
  return sqrt(x * x + y * y + z * z);
}

typedef struct { int32_t a, b, slot; } EdgeKey;

static int cmp_edge(const void* x, const void* y) {
  const EdgeKey* p = (const EdgeKey*)x;
  const EdgeKey* q = (const EdgeKey*)y;
  if (p->a != q->a) return p->a < q->a ? -1 : 1;
  if (p->b != q->b) return p->b < q->b ? -1 : 1;
  return p->slot < q->slot ? -1 : (p->slot > q->slot);
}

static int mesh_init(GMesh* m, int32_t nv, const float* pts, int32_t nf, const int32_t* f) {
  memset(m, 0, sizeof(*m));
  m->nv = nv;
  m->nf = nf;
  m->f = f;
  m->p = (double*)malloc(sizeof(double) * 3 * (size_t)nv);
  m->nbr = (int32_t*)malloc(sizeof(int32_t) * 3 * (size_t)nf);
  m->nbr_e = (int32_t*)malloc(sizeof(int32_t) * 3 * (size_t)nf);
  m->len = (double*)malloc(sizeof(double) * 3 * (size_t)nf);
  m->vf_off = (int64_t*)calloc((size_t)nv + 1, sizeof(int64_t));
  m->vf = (int32_t*)malloc(sizeof(int32_t) * 3 * (size_t)nf);
  m->saddle = (uint8_t*)calloc((size_t)nv, 1);
  EdgeKey* ek = (EdgeKey*)malloc(sizeof(EdgeKey) * 3 * (size_t)nf);
  double* angle = (double*)calloc((size_t)nv, sizeof(double));
  if (!m->p || !m->nbr || !m->nbr_e || !m->len || !m->vf_off || !m->vf || !m->saddle || !ek || !angle) return -1;
  for (int64_t i = 0; i < 3 * (int64_t)nv; ++i) m->p[i] = (double)pts[i];
  for (int32_t t = 0; t < nf; ++t) {
    for (int e = 0; e < 3; ++e) {
      const int32_t a = f[3 * t + e], b = f[3 * t + (e + 1) % 3];
      if (a < 0 || a >= nv || b < 0 || b >= nv || a == b) return -2;
      m->len[3 * t + e] = glen(m->p + 3 * a, m->p + 3 * b);
      ek[3 * t + e].a = a < b ? a : b;
      ek[3 * t + e].b = a < b ? b : a;
      ek[3 * t + e].slot = 3 * t + e;
      m->nbr[3 * t + e] = -1;
      m->nbr_e[3 * t + e] = -1;
      m->vf_off[a + 1]++;
    }
  }
  qsort(ek, 3 * (size_t)nf, sizeof(EdgeKey), cmp_edge);
  for (int64_t i = 0; i + 1 < 3 * (int64_t)nf; ++i) {
    if (ek[i].a == ek[i + 1].a && ek[i].b == ek[i + 1].b) {
      if (i + 2 < 3 * (int64_t)nf && ek[i + 2].a == ek[i].a && ek[i + 2].b == ek[i].b) return -3; /* non-manifold */
      const int32_t s0 = ek[i].slot, s1 = ek[i + 1].slot;
      m->nbr[s0] = s1 / 3;
      m->nbr_e[s0] = s1 % 3;
      m->nbr[s1] = s0 / 3;
      m->nbr_e[s1] = s0 % 3;
      ++i;
    }
  }
  for (int32_t v = 0; v < nv; ++v) m->vf_off[v + 1] += m->vf_off[v];
  int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)nv);
  if (!fill) return -1;
  memcpy(fill, m->vf_off, sizeof(int64_t) * (size_t)nv);
  for (int32_t t = 0; t < nf; ++t) {
    for (int e = 0; e < 3; ++e) {
      const int32_t v = f[3 * t + e];
      m->vf[fill[v]++] = t;
      /* corner angle at v between its two edges in face t */
      const double lo = m->len[3 * t + (e + 1) % 3]; /* opposite edge */
      const double l1 = m->len[3 * t + e], l2 = m->len[3 * t + (e + 2) % 3];
      double c = (l1 * l1 + l2 * l2 - lo * lo) / (2.0 * l1 * l2);
      c = c > 1.0 ? 1.0 : (c < -1.0 ? -1.0 : c);
      angle[v] += acos(c);
      if (m->nbr[3 * t + e] < 0) {
        m->saddle[f[3 * t + e]] = 1;
        m->saddle[f[3 * t + (e + 1) % 3]] = 1;
      }
    }
  }
  for (int32_t v = 0; v < nv; ++v)
    if (angle[v] > GEO_TWO_PI - 1e-5) m->saddle[v] = 1;
  free(fill);
  free(ek);
  free(angle);
  return 0;
}

static void mesh_free(GMesh* m) {
  free(m->p);
  free(m->nbr);
  free(m->nbr_e);
  free(m->len);
  free(m->vf_off);
  free(m->vf);
  free(m->saddle);
}

static int heap_push(GState* s, double key, int32_t idx, int32_t vert) {
  if (s->nh == s->ch) {
    s->ch = s->ch ? 2 * s->ch : 1024;
    GItem* n = (GItem*)realloc(s->h, sizeof(GItem) * (size_t)s->ch);
    if (!n) return -1;
    s->h = n;
  }
  int64_t i = s->nh++;
  while (i > 0) {
    const int64_t up = (i - 1) / 2;
    if (s->h[up].key <= key) break;
    s->h[i] = s->h[up];
    i = up;
  }
  s->h[i].key = key;
  s->h[i].idx = idx;
  s->h[i].vert = vert;
  return 0;
}

static GItem heap_pop(GState* s) {
  GItem top = s->h[0];
  const GItem last = s->h[--s->nh];
  int64_t i = 0;
  for (;;) {
    int64_t c = 2 * i + 1;
    if (c >= s->nh) break;
    if (c + 1 < s->nh && s->h[c + 1].key < s->h[c].key) ++c;
    if (s->h[c].key >= last.key) break;
    s->h[i] = s->h[c];
    i = c;
  }
  if (s->nh > 0) s->h[i] = last;
  return top;
}

static int touch(GState* s, int32_t v) {
  if (s->d[v] == INFINITY && s->done[v] == INFINITY) {
    if (s->nt == s->ct) {
      s->ct = s->ct ? 2 * s->ct : 1024;
      int32_t* n = (int32_t*)realloc(s->touched, sizeof(int32_t) * (size_t)s->ct);
      if (!n) return -1;
      s->touched = n;
    }
    s->touched[s->nt++] = v;
  }
  return 0;
}

/* d(v) = min(d(v), dv); a pseudo-source whose distance fell is queued */
static int reach(const GMesh* m, GState* s, int32_t v, double dv, double max_dist) {
  if (!(dv < s->d[v])) return 0;
  if (touch(s, v)) return -1;
  s->d[v] = dv;
  if (m->saddle[v] && dv <= max_dist) return heap_push(s, dv, v, 1);
  return 0;
}

/* distance from (sx, sy) to the segment [t0, t1] of the x axis */
static double seg_dist(double sx, double sy, double t0, double t1) {
  const double x = sx < t0 ? t0 - sx : (sx > t1 ? sx - t1 : 0.0);
  return sqrt(x * x + sy * sy);
}

/* a window on local edge e of face t (propagating into t) */
static int push_window(const GMesh* m, GState* s, int32_t t, int32_t e, double b0, double b1, double sx,
                       double sy, double sigma, double max_dist) {
  const double L = m->len[3 * t + e];
  if (b0 < 0.0) b0 = 0.0;
  if (b1 > L) b1 = L;
  if (!(b1 - b0 > 1e-12 * L)) return 0;
  const double key = sigma + seg_dist(sx, sy, b0, b1);
  if (key > max_dist) return 0;
  /* end-vertex filter: P = f_e at t = 0, Q = f_{e+1} at t = L */
  const double dP = s->d[m->f[3 * t + e]], dQ = s->d[m->f[3 * t + (e + 1) % 3]];
  const double far = sigma + hypot(sx - b1, sy), near = sigma + hypot(sx - b0, sy);
  if (far > dP + b1 || near > dQ + (L - b0)) return 0;
  if (s->nw == s->cw) {
    s->cw = s->cw ? 2 * s->cw : 1024;
    GWin* n = (GWin*)realloc(s->w, sizeof(GWin) * (size_t)s->cw);
    if (!n) return -1;
    s->w = n;
  }
  GWin* w = s->w + s->nw;
  w->face = t;
  w->edge = e;
  w->b0 = b0;
  w->b1 = b1;
  w->sx = sx;
  w->sy = sy;
  w->sigma = sigma;
  return heap_push(s, key, (int32_t)s->nw++, 0);
}

/* the child of a window crossing face t on the edge from 2-D point pa (mesh
 * vertex va) to pb (vertex vb), covering the segment [q0, q1] of that edge;
 * pthird is the face's third vertex, on the far side from the neighbour */
static int child(const GMesh* m, GState* s, int32_t t, int32_t le, const double* pa, const double* pb,
                 const double* pthird, const double* q0, const double* q1, double sx, double sy, double sigma,
                 double max_dist) {
  const int32_t g = m->nbr[3 * t + le];
  if (g < 0) return 0;
  const int32_t ge = m->nbr_e[3 * t + le];
  const int32_t gp = m->f[3 * g + ge];
  const int32_t va = m->f[3 * t + le];
  /* the neighbour's edge runs P -> Q; P is va or the other end */
  const double* pP = (gp == va) ? pa : pb;
  const double* pQ = (gp == va) ? pb : pa;
  double ux = pQ[0] - pP[0], uy = pQ[1] - pP[1];
  const double ul = hypot(ux, uy);
  ux /= ul;
  uy /= ul;
  double nx = -uy, ny = ux;
  if (nx * (pthird[0] - pP[0]) + ny * (pthird[1] - pP[1]) > 0.0) {
    nx = -nx;
    ny = -ny;
  }
  const double s2x = (sx - pP[0]) * ux + (sy - pP[1]) * uy;
  const double s2y = (sx - pP[0]) * nx + (sy - pP[1]) * ny;
  if (!(s2y < 0.0)) return 0;  /* the image lies on the edge's line: no area behind it */
  double t0 = (q0[0] - pP[0]) * ux + (q0[1] - pP[1]) * uy;
  double t1 = (q1[0] - pP[0]) * ux + (q1[1] - pP[1]) * uy;
  if (t0 > t1) {
    const double x = t0;
    t0 = t1;
    t1 = x;
  }
  return push_window(m, s, g, ge, t0, t1, s2x, s2y, sigma, max_dist);
}

/* point where the line from s through (x, 0) meets the line through a, b */
static void hit(double sx, double sy, double x, const double* a, const double* b, double* out) {
  const double dx = x - sx, dy = -sy;
  const double ex = b[0] - a[0], ey = b[1] - a[1];
  const double den = ex * dy - ey * dx;
  const double mu = ((sx - a[0]) * dy - (sy - a[1]) * dx) / den;
  const double muc = mu < 0.0 ? 0.0 : (mu > 1.0 ? 1.0 : mu);
  out[0] = a[0] + muc * ex;
  out[1] = a[1] + muc * ey;
}

static int propagate_window(const GMesh* m, GState* s, const GWin* w, double max_dist) {
  const int32_t t = w->face, e = w->edge;
  const int32_t vc = m->f[3 * t + (e + 2) % 3];
  const double L = m->len[3 * t + e];
  const double la = m->len[3 * t + (e + 2) % 3]; /* C -> A */
  const double lb = m->len[3 * t + (e + 1) % 3]; /* B -> C */
  const double cx = (L * L + la * la - lb * lb) / (2.0 * L);
  const double cy2 = la * la - cx * cx;
  const double cy = cy2 > 0.0 ? sqrt(cy2) : 0.0;
  const double A[2] = {0.0, 0.0}, B[2] = {L, 0.0}, C[2] = {cx, cy};
  const double sx = w->sx, sy = w->sy;
  const double xc = sx + (cx - sx) * (-sy) / (cy - sy); /* where the line s -> C crosses the edge */
  if (xc >= w->b0 && xc <= w->b1 && reach(m, s, vc, w->sigma + hypot(cx - sx, cy - sy), max_dist)) return -1;
  double q0[2], q1[2];
  if (w->b0 < xc) { /* edge C -> A: local edge e + 2 */
    hit(sx, sy, w->b0, A, C, q0);
    if (w->b1 < xc) hit(sx, sy, w->b1, A, C, q1);
    else {
      q1[0] = cx;
      q1[1] = cy;
    }
    if (child(m, s, t, (e + 2) % 3, C, A, B, q0, q1, sx, sy, w->sigma, max_dist)) return -1;
  }
  if (w->b1 > xc) { /* edge B -> C: local edge e + 1 */
    if (w->b0 > xc) hit(sx, sy, w->b0, B, C, q0);
    else {
      q0[0] = cx;
      q0[1] = cy;
    }
    hit(sx, sy, w->b1, B, C, q1);
    if (child(m, s, t, (e + 1) % 3, B, C, A, q0, q1, sx, sy, w->sigma, max_dist)) return -1;
  }
  return 0;
}

/* a (pseudo-)source u at distance du: its neighbours along the edges, and a
 * window on the edge opposite u in every face around it, crossing into the
 * face beyond that edge */
static int expand_vertex(const GMesh* m, GState* s, int32_t u, double du, double max_dist) {
  for (int64_t k = m->vf_off[u]; k < m->vf_off[u + 1]; ++k) {
    const int32_t t = m->vf[k];
    int c = 0;
    while (m->f[3 * t + c] != u) ++c;
    const int32_t e = (c + 1) % 3; /* opposite edge: f_{c+1} -> f_{c+2} */
    const int32_t v1 = m->f[3 * t + e], v2 = m->f[3 * t + (e + 1) % 3];
    const double l1 = m->len[3 * t + c];            /* u -> v1 */
    const double l2 = m->len[3 * t + (c + 2) % 3];  /* v2 -> u */
    if (reach(m, s, v1, du + l1, max_dist) || reach(m, s, v2, du + l2, max_dist)) return -1;
    const int32_t g = m->nbr[3 * t + e];
    if (g < 0) continue;
    const int32_t ge = m->nbr_e[3 * t + e];
    const double L = m->len[3 * t + e];
    /* in the frame of g's edge P -> Q, u lies behind the edge (y < 0) */
    const int32_t gp = m->f[3 * g + ge];
    const double dPu = (gp == v1) ? l1 : l2, dQu = (gp == v1) ? l2 : l1;
    const double x = (L * L + dPu * dPu - dQu * dQu) / (2.0 * L);
    const double y2 = dPu * dPu - x * x;
    const double y = -(y2 > 0.0 ? sqrt(y2) : 0.0);
    if (y < 0.0 && push_window(m, s, g, ge, 0.0, L, x, y, du, max_dist)) return -1;
  }
  return 0;
}

static int run_source(const GMesh* m, GState* s, int32_t src, double max_dist) {
  s->nw = 0;
  s->nh = 0;
  if (touch(s, src)) return -1;
  s->d[src] = 0.0;
  s->done[src] = 0.0;
  if (expand_vertex(m, s, src, 0.0, max_dist)) return -1;
  while (s->nh > 0) {
    const GItem it = heap_pop(s);
    if (it.key > max_dist) break;
    if (it.vert) {
      const int32_t v = it.idx;
      if (it.key > s->d[v] || s->done[v] <= it.key) continue;  /* stale, or expanded already */
      s->done[v] = it.key;
      if (expand_vertex(m, s, v, it.key, max_dist)) return -1;
    } else {
      const GWin w = s->w[it.idx];
      if (propagate_window(m, s, &w, max_dist)) return -1;
    }
  }
  return 0;
}

static int cmp_i32(const void* a, const void* b) {
  const int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
  return (x > y) - (x < y);
}

/* returns 0, -1 (allocation), -2/-3 (bad mesh), -4 (output capacity) */
int oracle_geodesic_lists(int32_t nv, const float* pts, int32_t nf, const int32_t* faces, double threshold,
                          int32_t only_greater, int32_t src_lo, int32_t src_hi, int64_t cap, int32_t* out_i,
                          int32_t* out_j, double* out_d, int64_t* n_out) {
  GMesh m;
  int rc = mesh_init(&m, nv, pts, nf, faces);
  GState s;
  memset(&s, 0, sizeof(s));
  int64_t n = 0;
  const double max_dist = threshold + 1e-10; /* adjacency.pyx:54 */
  if (!rc) {
    s.d = (double*)malloc(sizeof(double) * (size_t)nv);
    s.done = (double*)malloc(sizeof(double) * (size_t)nv);
    if (!s.d || !s.done) rc = -1;
  }
  if (!rc)
    for (int32_t v = 0; v < nv; ++v) s.d[v] = s.done[v] = INFINITY;
  for (int32_t src = src_lo; !rc && src < src_hi; ++src) {
    rc = run_source(&m, &s, src, max_dist);
    if (rc) break;
    qsort(s.touched, (size_t)s.nt, sizeof(int32_t), cmp_i32);
    for (int64_t k = 0; k < s.nt; ++k) {
      const int32_t j = s.touched[k];
      if (j == src || (only_greater && j < src) || !(s.d[j] < threshold)) continue;
      if (n >= cap) {
        rc = -4;
        break;
      }
      out_i[n] = src;
      out_j[n] = j;
      out_d[n] = s.d[j];
      ++n;
    }
    for (int64_t k = 0; k < s.nt; ++k) s.d[s.touched[k]] = s.done[s.touched[k]] = INFINITY;
    s.nt = 0;
  }
  *n_out = n;
  free(s.w);
  free(s.h);
  free(s.d);
  free(s.done);
  free(s.touched);
  mesh_free(&m);
  return rc;
}
