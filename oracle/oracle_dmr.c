/* CPU oracle for Delaunay mesh refinement -- TEST INFRASTRUCTURE.
 *
 * Restates LonestarGPU DMR (lonestar/apps/dmr/kernel/dmr_common.cl and
 * dmr_port_kernel.cl:35-188, host loop dmr_port.cpp:160-316) in serial C,
 * with the schedule made deterministic:
 *
 *  * a round's worklist is the previous round's repushed items in the
 *    order they were processed, then the bad triangles among the elements
 *    the round created, in element order (dmr_port.cpp:284-306, where the
 *    reference's order comes from atomics);
 *  * a round is processed in chunks of `chunk` items (one per thread of a
 *    launch); in a chunk every item builds its cavity from the mesh as the
 *    chunk found it, claims the cavity and its outside neighbours, and the
 *    lowest item claiming an element owns it (the reference's owner store +
 *    atomic_min, dmr_port_kernel.cl:76-112); an item that owns everything it
 *    claimed commits;
 *  * the committing items take node and element slots in item order (the
 *    reference: atomic_add, dmr_port_kernel.cl:137-141).
 *
 * With chunk = 1 this is the reference's own sequential schedule; the
 * reference's kernels run through oracle/refshim pin it there.  Geometry
 * is the reference's double arithmetic, operation for operation (compiled
 * without floating-point contraction), with rsqrt(v) read as 1 / sqrt(v)
 * and cos(30 degrees) as the correctly rounded double.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NONE 1234567890u /* INVALIDID, dmr_common.cl:49 */
#define CAVLEN 256       /* dmr_common.cl:58-59 */
#define BCLEN 1024
static const double kCos30 = 0x1.bb67ae8584cabp-1; /* cos(30 * (PI / 180)) */

typedef struct {
  double *x, *y;
  uint32_t *el, *nb; /* 3 per element */
  uint8_t *del, *bad;
  uint32_t nn, ne, maxn, maxe;
} Mesh;

static int is_seg(const uint32_t* e) { return e[2] == NONE; }

/* dmr_common.cl:107-117 */
static double dist2(double ax, double ay, double bx, double by) {
  double dx = ax - bx;
  double dy = ay - by;
  return dx * dx + dy * dy;
}

/* angleLT, dmr_common.cl:119-142: is the angle at c below 30 degrees */
static int angle_lt(const Mesh* m, uint32_t a, uint32_t b, uint32_t c) {
  double vax = m->x[a] - m->x[c];
  double vay = m->y[a] - m->y[c];
  double vbx = m->x[b] - m->x[c];
  double vby = m->y[b] - m->y[c];
  double dp = vax * vbx + vay * vby;
  if (dp < 0.0) return 0;
  double da = dist2(m->x[a], m->y[a], m->x[c], m->y[c]);
  double db = dist2(m->x[b], m->y[b], m->x[c], m->y[c]);
  double cc = dp * (1.0 / sqrt(da * db));
  return cc > kCos30;
}

/* angleOB, dmr_common.cl:189-199: is the angle at c obtuse */
static int angle_ob(const Mesh* m, uint32_t a, uint32_t b, uint32_t c) {
  double vax = m->x[a] - m->x[c];
  double vay = m->y[a] - m->y[c];
  double vbx = m->x[b] - m->x[c];
  double vby = m->y[b] - m->y[c];
  double dp = vax * vbx + vay * vby;
  return dp < 0.0;
}

static int tri_bad(const Mesh* m, const uint32_t* e) {
  return angle_lt(m, e[0], e[1], e[2]) || angle_lt(m, e[2], e[0], e[1]) ||
         angle_lt(m, e[1], e[2], e[0]);
}

static int has_node(const uint32_t* e, uint32_t n) { return e[0] == n || e[1] == n || e[2] == n; }

/* find_shared_edge, dmr_common.cl:201-212 (unset entries stay NONE) */
static void shared_edge(const uint32_t* e1, const uint32_t* e2, uint32_t* se) {
  int sc = 0;
  se[0] = se[1] = NONE;
  if (has_node(e2, e1[0])) se[sc++] = e1[0];
  if (has_node(e2, e1[1])) se[sc++] = e1[1];
  if (!is_seg(e1) && has_node(e2, e1[2]) && sc < 2) se[sc++] = e1[2];
}

/* does neighbour n of triangle e share the edge facing node ob */
static int faces(const Mesh* m, const uint32_t* e, uint32_t n, uint32_t ob) {
  if (n == NONE) return 0;
  uint32_t se[2];
  shared_edge(e, m->el + 3 * (size_t)n, se);
  return se[0] == ob || se[1] == ob;
}

/* opposite, dmr_common.cl:214-256: a triangle obtuse at some node hands its
 * refinement to the neighbour across the edge facing that node */
static uint32_t opposite(const Mesh* m, uint32_t t) {
  const uint32_t* e = m->el + 3 * (size_t)t;
  if (is_seg(e)) return t;
  uint32_t ob;
  if (angle_ob(m, e[0], e[1], e[2])) ob = e[2];
  else if (angle_ob(m, e[2], e[0], e[1])) ob = e[1];
  else if (angle_ob(m, e[1], e[2], e[0])) ob = e[0];
  else return t;
  const uint32_t* nb = m->nb + 3 * (size_t)t;
  uint32_t cand = nb[0];
  /* a missing neighbour (NONE) shares no edge; the reference would read
   * element NONE here, past its arrays, and the caller rejects a NONE
   * hand-off instead */
  if (faces(m, e, nb[0], ob)) {
    cand = nb[1];
    if (faces(m, e, nb[1], ob)) cand = nb[2];
  }
  return cand;
}

/* dmr_common.cl:258-276 */
static void circumcenter(double Ax, double Ay, double Bx, double By, double Cx, double Cy,
                         double* ccx, double* ccy) {
  double D = 2 * (Ax * (By - Cy) + Bx * (Cy - Ay) + Cx * (Ay - By));
  *ccx = ((Ax * Ax + Ay * Ay) * (By - Cy) + (Bx * Bx + By * By) * (Cy - Ay) +
          (Cx * Cx + Cy * Cy) * (Ay - By)) / D;
  *ccy = ((Ax * Ax + Ay * Ay) * (Cx - Bx) + (Bx * Bx + By * By) * (Ax - Cx) +
          (Cx * Cx + Cy * Cy) * (Bx - Ax)) / D;
}

/* dmr_common.cl:278-287 */
static double ccw(double pax, double pay, double pbx, double pby, double pcx, double pcy) {
  double detleft = (pax - pcx) * (pby - pcy);
  double detright = (pay - pcy) * (pbx - pcx);
  return detleft - detright;
}

/* gincircle, dmr_common.cl:290-320 */
static double incircle(double ax, double ay, double bx, double by, double cx, double cy, double px,
                       double py) {
  double apx = ax - px, bpx = bx - px, cpx = cx - px;
  double apy = ay - py, bpy = by - py, cpy = cy - py;
  double bpxcpy = bpx * cpy, cpxbpy = cpx * bpy;
  double alift = apx * apx + apy * apy;
  double cpxapy = cpx * apy, apxcpy = apx * cpy;
  double blift = bpx * bpx + bpy * bpy;
  double apxbpy = apx * bpy, bpxapy = bpx * apy;
  double clift = cpx * cpx + cpy * cpy;
  return alift * (bpxcpy - cpxbpy) + blift * (cpxapy - apxcpy) + clift * (apxbpy - bpxapy);
}

/* encroached, dmr_common.cl:322-356: does the new point lie in element t's
 * circumcircle (triangle) or diametral circle (segment) */
static int encroached(const Mesh* m, uint32_t t, const uint32_t* root, double cx, double cy,
                      int* seg) {
  if (t == NONE) return 0;
  const uint32_t* e = m->el + 3 * (size_t)t;
  const double* X = m->x;
  const double* Y = m->y;
  if (is_seg(e)) {
    *seg = 1;
    uint32_t nsp = root[0] == e[0] ? (root[1] == e[1] ? root[2] : root[1]) : root[0];
    if ((ccw(X[e[0]], Y[e[0]], X[e[1]], Y[e[1]], X[nsp], Y[nsp]) > 0.0) !=
        (ccw(X[e[0]], Y[e[0]], X[e[1]], Y[e[1]], cx, cy) > 0.0))
      return 1;
    double mx = (X[e[0]] + X[e[1]]) / 2;
    double my = (Y[e[0]] + Y[e[1]]) / 2;
    double r2 = dist2(mx, my, X[e[0]], Y[e[0]]);
    return dist2(cx, cy, mx, my) < r2;
  }
  return incircle(X[e[0]], Y[e[0]], X[e[1]], Y[e[1]], X[e[2]], Y[e[2]], cx, cy) > 0.0;
}

typedef struct {
  uint32_t cav[CAVLEN], nc;
  uint32_t bnd[BCLEN], bc;
  double cx, cy;
} Cavity;

/* add_to_cavity / add_to_boundary, dmr_common.cl:358-387 */
static int cav_add(Cavity* k, uint32_t t) {
  for (uint32_t i = 0; i < k->nc; ++i)
    if (k->cav[i] == t) return 0;
  if (k->nc >= CAVLEN) return -1;
  k->cav[k->nc++] = t;
  return 0;
}
static int bnd_add(Cavity* k, uint32_t s1, uint32_t s2, uint32_t src, uint32_t dst) {
  for (uint32_t i = 0; i < k->bc; i += 4)
    if ((s1 == k->bnd[i] && s2 == k->bnd[i + 1]) || (s1 == k->bnd[i + 1] && s2 == k->bnd[i])) return 0;
  if (k->bc + 4 > BCLEN) return -1;
  k->bnd[k->bc++] = s1;
  k->bnd[k->bc++] = s2;
  k->bnd[k->bc++] = src;
  k->bnd[k->bc++] = dst;
  return 0;
}

/* build_cavity, dmr_common.cl:390-446: 1 built, 0 restart from the
 * encroached segment now in cav[0], -1 capacity */
static int build_cavity(const Mesh* m, Cavity* k) {
  uint32_t root[3];
  memcpy(root, m->el + 3 * (size_t)k->cav[0], sizeof root);
  if (is_seg(root)) {
    k->cx = (m->x[root[0]] + m->x[root[1]]) / 2;
    k->cy = (m->y[root[0]] + m->y[root[1]]) / 2;
  } else {
    circumcenter(m->x[root[0]], m->y[root[0]], m->x[root[1]], m->y[root[1]], m->x[root[2]],
                 m->y[root[2]], &k->cx, &k->cy);
  }
  for (uint32_t ce = 0; ce < k->nc; ++ce) {
    uint32_t nbs[3];
    memcpy(nbs, m->nb + 3 * (size_t)k->cav[ce], sizeof nbs);
    for (int i = 0; i < 3; ++i) {
      const uint32_t n = nbs[i];
      if (n == k->cav[0] || n == NONE) continue;
      int seg = 0;
      if (!(is_seg(root) && is_seg(m->el + 3 * (size_t)n)) &&
          encroached(m, n, root, k->cx, k->cy, &seg)) {
        if (!seg) {
          if (cav_add(k, n)) return -1;
        } else {
          k->cav[0] = n;
          k->nc = 1;
          k->bc = 0;
          return 0;
        }
      } else {
        uint32_t se[2];
        shared_edge(m->el + 3 * (size_t)k->cav[ce], m->el + 3 * (size_t)n, se);
        if (bnd_add(k, se[0], se[1], n, k->cav[ce])) return -1;
      }
    }
  }
  return 1;
}

/* addneighbour, dmr_common.cl:527-534 */
static void add_neighbour(uint32_t* nb, uint32_t t) {
  if (nb[0] == t || nb[1] == t || nb[2] == t) return;
  if (nb[0] == NONE) { nb[0] = t; return; }
  if (nb[1] == NONE) { nb[1] = t; return; }
  if (nb[2] == NONE) { nb[2] = t; return; }
}

/* adjacent, dmr_common.cl:510-525 */
static int adjacent(const uint32_t* e1, const uint32_t* e2) {
  int sc = has_node(e2, e1[0]) + has_node(e2, e1[1]);
  if (!is_seg(e1)) sc += has_node(e2, e1[2]);
  return sc == 2;
}

/* find_neighbours_cpu (dmr.h:55-104): elements in index order, each edge
 * of a triangle (one for a segment) between sorted node ids; an edge seen
 * a second time links the two elements. */
typedef struct {
  uint64_t* key;
  uint32_t* val;
  uint8_t* state; /* 0 empty, 1 full, 2 erased */
  size_t cap;
} EdgeMap;

static size_t edge_slot(const EdgeMap* h, uint64_t k) {
  uint64_t z = k * 0x9E3779B97F4A7C15ull;
  return (size_t)(z ^ (z >> 29)) & (h->cap - 1);
}

int orc_dmr_neighbours(uint32_t ne, const uint32_t* el, uint32_t* nb) {
  EdgeMap h;
  h.cap = 16;
  while (h.cap < 4 * (size_t)ne + 16) h.cap <<= 1;
  h.key = (uint64_t*)malloc(h.cap * sizeof(uint64_t));
  h.val = (uint32_t*)malloc(h.cap * sizeof(uint32_t));
  h.state = (uint8_t*)calloc(h.cap, 1);
  if (!h.key || !h.val || !h.state) {
    free(h.key); free(h.val); free(h.state);
    return -2;
  }
  for (uint32_t t = 0; t < ne; ++t) {
    uint32_t* n = nb + 3 * (size_t)t;
    n[0] = n[1] = n[2] = NONE;
    uint32_t s[3] = {el[3 * (size_t)t], el[3 * (size_t)t + 1], el[3 * (size_t)t + 2]};
    uint32_t tmp;
    if (s[0] > s[1]) { tmp = s[0]; s[0] = s[1]; s[1] = tmp; }
    if (s[1] > s[2]) { tmp = s[1]; s[1] = s[2]; s[2] = tmp; }
    if (s[0] > s[1]) { tmp = s[0]; s[0] = s[1]; s[1] = tmp; }
    const uint64_t edges[3] = {((uint64_t)s[0] << 32) | s[1], ((uint64_t)s[1] << 32) | s[2],
                               ((uint64_t)s[0] << 32) | s[2]};
    const int maxn = is_seg(el + 3 * (size_t)t) ? 1 : 3;
    for (int i = 0; i < maxn; ++i) {
      size_t p = edge_slot(&h, edges[i]), tomb = (size_t)-1;
      for (;; p = (p + 1) & (h.cap - 1)) {
        if (h.state[p] == 0) break;
        if (h.state[p] == 2) {
          if (tomb == (size_t)-1) tomb = p;
          continue;
        }
        if (h.key[p] == edges[i]) break;
      }
      if (h.state[p] == 1) {
        const uint32_t other = h.val[p];
        add_neighbour(nb + 3 * (size_t)other, t);
        add_neighbour(n, other);
        h.state[p] = 2;
      } else {
        if (tomb != (size_t)-1) p = tomb;
        h.state[p] = 1;
        h.key[p] = edges[i];
        h.val[p] = t;
      }
    }
  }
  free(h.key); free(h.val); free(h.state);
  return 0;
}

/* add_triangle, dmr_common.cl:475-508: counter-clockwise node order, the
 * outside neighbour nb1 re-pointed from the deleted oldt */
static void add_triangle(Mesh* m, uint32_t n1, uint32_t n2, uint32_t n3, uint32_t nb1,
                         uint32_t oldt, uint32_t ndx) {
  uint32_t* e = m->el + 3 * (size_t)ndx;
  if (ccw(m->x[n1], m->y[n1], m->x[n2], m->y[n2], m->x[n3], m->y[n3]) > 0) {
    e[0] = n1; e[1] = n2; e[2] = n3;
  } else {
    e[0] = n3; e[1] = n2; e[2] = n1;
  }
  m->bad[ndx] = 0;
  m->del[ndx] = 0;
  uint32_t* nb = m->nb + 3 * (size_t)ndx;
  nb[0] = nb1;
  nb[1] = nb[2] = NONE;
  uint32_t* o = m->nb + 3 * (size_t)nb1;
  if (o[0] == oldt) o[0] = ndx;
  else if (o[1] == oldt) o[1] = ndx;
  else o[2] = ndx;
}

/* add_segment, dmr_common.cl:462-473 */
static void add_segment(Mesh* m, uint32_t n1, uint32_t n2, uint32_t ndx) {
  uint32_t* e = m->el + 3 * (size_t)ndx;
  e[0] = n1; e[1] = n2; e[2] = NONE;
  m->bad[ndx] = 0;
  m->del[ndx] = 0;
  uint32_t* nb = m->nb + 3 * (size_t)ndx;
  nb[0] = nb[1] = nb[2] = NONE;
}

/* A chunk's cavities, stored compactly: item t's cavity elements are
 * arena[off[t] .. off[t] + nc[t]), its boundary records (4 words each)
 * follow them. */
typedef struct {
  uint32_t* arena;
  size_t len, cap;
} Arena;

static int arena_put(Arena* a, const uint32_t* v, size_t n) {
  if (a->len + n > a->cap) {
    size_t c = a->cap ? a->cap : 4096;
    while (c < a->len + n) c *= 2;
    uint32_t* p = (uint32_t*)realloc(a->arena, c * sizeof(uint32_t));
    if (!p) return -1;
    a->arena = p;
    a->cap = c;
  }
  memcpy(a->arena + a->len, v, n * sizeof(uint32_t));
  a->len += n;
  return 0;
}

int orc_dmr_refine(const double* x0, const double* y0, uint32_t nnodes, const uint32_t* el0,
                   uint32_t nelements, uint32_t maxfactor, uint32_t chunk, double* x, double* y,
                   uint32_t* el, uint32_t* nb, uint8_t* isdel, uint32_t* counts) {
  if (!chunk || !nnodes || !nelements || maxfactor < 2) return -1;
  Mesh m;
  m.maxn = (maxfactor / 2) * nnodes; /* meshfiles.h:27, shmesh.h:48 */
  m.maxe = maxfactor * nelements;    /* meshfiles.h:67 */
  m.nn = nnodes;
  m.ne = nelements;
  m.x = x;
  m.y = y;
  m.el = el;
  m.nb = nb;
  m.del = isdel;
  const uint32_t cmax = chunk < m.maxe ? chunk : m.maxe; /* items of one chunk */
  m.bad = (uint8_t*)calloc(m.maxe, 1);
  uint32_t* wl = (uint32_t*)malloc(sizeof(uint32_t) * m.maxe);
  uint32_t* nwl = (uint32_t*)malloc(sizeof(uint32_t) * m.maxe);
  uint32_t* own = (uint32_t*)malloc(sizeof(uint32_t) * m.maxe);
  uint32_t* stamp = (uint32_t*)calloc(m.maxe, sizeof(uint32_t));
  size_t* off = (size_t*)malloc(sizeof(size_t) * cmax);
  uint32_t* ncs = (uint32_t*)malloc(sizeof(uint32_t) * cmax);
  uint32_t* bcs = (uint32_t*)malloc(sizeof(uint32_t) * cmax);
  double* cxs = (double*)malloc(sizeof(double) * cmax);
  double* cys = (double*)malloc(sizeof(double) * cmax);
  uint8_t* act = (uint8_t*)malloc(cmax);
  Cavity* k = (Cavity*)malloc(sizeof(Cavity));
  Arena ar = {NULL, 0, 0};
  int rc = 0;
  if (!m.bad || !wl || !nwl || !own || !stamp || !off || !ncs || !bcs || !cxs || !cys || !act || !k) {
    rc = -2;
    goto out;
  }
  memcpy(x, x0, sizeof(double) * nnodes);
  memcpy(y, y0, sizeof(double) * nnodes);
  memcpy(el, el0, sizeof(uint32_t) * 3 * (size_t)nelements);
  memset(isdel, 0, nelements);
  if (orc_dmr_neighbours(nelements, el, nb)) { rc = -2; goto out; }
  /* check_triangles from 0 (dmr_common.cl:145-187) */
  uint32_t nw = 0;
  for (uint32_t t = 0; t < m.ne; ++t) {
    const uint32_t* e = el + 3 * (size_t)t;
    if (is_seg(e)) continue;
    m.bad[t] = (uint8_t)tri_bad(&m, e);
    if (m.bad[t]) wl[nw++] = t;
  }
  uint32_t rounds = 0, steps = 0, refined = 0, cur_stamp = 0;
  while (nw) {
    if (++rounds > 100000) { rc = -4; goto out; }
    const uint32_t last = m.ne;
    uint32_t nn2 = 0;
    for (uint32_t s = 0; s < nw; s += chunk) {
      const uint32_t cnt = nw - s < chunk ? nw - s : chunk;
      ++steps;
      ++cur_stamp;
      ar.len = 0;
      /* cavities from the chunk's mesh (dmr_port_kernel.cl:58-85), claims:
       * the lowest claiming item owns an element */
      for (uint32_t t = 0; t < cnt; ++t) {
        const uint32_t ele = wl[s + t];
        act[t] = ele < last && m.bad[ele] && !m.del[ele];
        if (!act[t]) continue;
        k->nc = 1;
        k->bc = 0;
        k->cav[0] = opposite(&m, ele);
        if (k->cav[0] == NONE) { rc = -6; goto out; } /* an obtuse triangle facing no neighbour */
        int r = build_cavity(&m, k);
        if (r == 0) r = build_cavity(&m, k);
        if (r < 0) { rc = -5; goto out; }
        off[t] = ar.len;
        ncs[t] = k->nc;
        bcs[t] = k->bc;
        cxs[t] = k->cx;
        cys[t] = k->cy;
        if (arena_put(&ar, k->cav, k->nc) || arena_put(&ar, k->bnd, k->bc)) { rc = -2; goto out; }
        for (uint32_t i = 0; i < k->nc + k->bc / 4; ++i) {
          const uint32_t c = i < k->nc ? k->cav[i] : k->bnd[4 * (i - k->nc) + 2];
          if (stamp[c] != cur_stamp) { stamp[c] = cur_stamp; own[c] = t; }
          else if (t < own[c]) own[c] = t;
        }
      }
      /* owners settled (dmr_port_kernel.cl:90-129); node and element slots
       * in item order; the commits write only what their items own */
      for (uint32_t t = 0; t < cnt; ++t) {
        if (!act[t]) continue;
        const uint32_t ele = wl[s + t];
        const uint32_t* cav = ar.arena + off[t];
        const uint32_t* bnd = cav + ncs[t];
        int win = 1;
        for (uint32_t i = 0; i < ncs[t] + bcs[t] / 4 && win; ++i)
          win = own[i < ncs[t] ? cav[i] : bnd[4 * (i - ncs[t]) + 2]] == t;
        if (!win) { nwl[nn2++] = ele; continue; }
        const uint32_t* root = el + 3 * (size_t)cav[0];
        const uint32_t ne_add = bcs[t] / 4 + (is_seg(root) ? 2u : 0u);
        if (m.nn + 1 > m.maxn || m.ne + ne_add > m.maxe) { rc = -3; goto out; }
        const uint32_t cnode = m.nn++;
        x[cnode] = cxs[t];
        y[cnode] = cys[t];
        const uint32_t first = m.ne;
        uint32_t nx = first;
        m.ne += ne_add;
        if (is_seg(root)) {
          const uint32_t r0 = root[0], r1 = root[1];
          add_segment(&m, r0, cnode, nx++);
          add_segment(&m, cnode, r1, nx++);
        }
        for (uint32_t i = 0; i < bcs[t]; i += 4)
          add_triangle(&m, bnd[i], bnd[i + 1], cnode, bnd[i + 2], bnd[i + 3], nx++);
        /* setup_neighbours, dmr_common.cl:538-555 */
        for (uint32_t i = first; i < nx; ++i)
          for (uint32_t j = i + 1; j < nx; ++j)
            if (adjacent(el + 3 * (size_t)i, el + 3 * (size_t)j)) {
              add_neighbour(nb + 3 * (size_t)i, j);
              add_neighbour(nb + 3 * (size_t)j, i);
            }
        int repush = 1;
        for (uint32_t i = 0; i < ncs[t]; ++i) {
          isdel[cav[i]] = 1;
          if (cav[i] == ele) repush = 0;
        }
        if (repush) nwl[nn2++] = ele;
        ++refined;
      }
    }
    /* check_triangles from `last` (dmr_port.cpp:284-297) */
    for (uint32_t t = last; t < m.ne; ++t) {
      const uint32_t* e = el + 3 * (size_t)t;
      if (isdel[t] || is_seg(e)) continue;
      if (!m.bad[t]) m.bad[t] = (uint8_t)tri_bad(&m, e);
      if (m.bad[t]) nwl[nn2++] = t;
    }
    uint32_t* tmp = wl;
    wl = nwl;
    nwl = tmp;
    nw = nn2;
  }
  counts[0] = m.nn;
  counts[1] = m.ne;
  counts[2] = rounds;
  counts[3] = steps;
  counts[4] = refined;
out:
  free(m.bad);
  free(wl);
  free(nwl);
  free(own);
  free(stamp);
  free(off);
  free(ncs);
  free(bcs);
  free(cxs);
  free(cys);
  free(act);
  free(k);
  free(ar.arena);
  return rc;
}

/* Bad triangles left among the live elements (the reference's final check,
 * dmr_port.cpp:327-353). */
uint32_t orc_dmr_count_bad(const double* x, const double* y, uint32_t ne, const uint32_t* el,
                           const uint8_t* isdel) {
  Mesh m;
  memset(&m, 0, sizeof m);
  m.x = (double*)x;
  m.y = (double*)y;
  uint32_t n = 0;
  for (uint32_t t = 0; t < ne; ++t) {
    const uint32_t* e = el + 3 * (size_t)t;
    if (isdel[t] || is_seg(e)) continue;
    n += (uint32_t)tri_bad(&m, e);
  }
  return n;
}
