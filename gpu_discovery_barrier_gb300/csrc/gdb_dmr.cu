// Delaunay mesh refinement (LonestarGPU DMR) as one persistent kernel.
//
// Replaces the reference's host loop (lonestar_gpu_opencl/apps/dmr/dmr_port.cpp:160-316),
// which launches the refine kernel (dmr_port_kernel.cl:37-188) over the
// worklist and check_triangles (dmr_common.cl:144-187) over the new
// elements until no bad triangle is left, with one launch and grid barriers
// between its phases.  The schedule is deterministic, so the refined mesh
// is the same on every run and for every launch shape:
//
//  * a round's worklist is the previous round's repushed items in the order
//    they were processed, then the bad triangles among the elements the
//    round created, in element order (the reference orders them by atomics);
//  * a round is processed in chunks of `chunk` items; every item of a chunk
//    builds its cavity from the mesh as the chunk found it and claims the
//    cavity and its outside neighbours; the lowest item claiming an element
//    owns it (the reference's owner store + atomic_min,
//    dmr_port_kernel.cl:76-112), and an item that owns everything it claimed
//    commits;
//  * the committing items take node and element slots in item order (the
//    reference takes them with atomic_add, dmr_port_kernel.cl:137-141).
//
// Per chunk: build + claim | barrier | ownership test and slot counts |
// barrier | prefix sums (CTA 0) | barrier | commit | barrier.  Per round
// after the chunks: bad-triangle test of the new elements | barrier |
// prefix sums of the per-CTA counts (CTA 0) | barrier | ordered append |
// barrier.
//
// The geometry is the reference's double arithmetic, operation for
// operation (dmr_common.cl:107-356), and this file is compiled without
// floating-point contraction, so the coordinates of the new nodes are the
// same bits as the serial restatement's; rsqrt(v) is computed as
// 1 / sqrt(v), both correctly rounded.
#include <algorithm>
#include <unordered_map>
#include <vector>

#include "gdb_internal.h"

namespace {

using namespace gdb;

constexpr uint32_t kNone = 1234567890u;  // INVALIDID, dmr_common.cl:49
constexpr uint32_t kCav = 256;           // cavity elements per item (dmr_common.cl:58)
constexpr uint32_t kBnd = 1024;          // boundary words per item (dmr_common.cl:59)
constexpr int kBlock = 256;
constexpr uint32_t kMaxRounds = 100000;

struct DmrMesh {
  double* x;
  double* y;
  uint32_t* el;   // 3 per element; a segment's third node is kNone
  uint32_t* nb;   // 3 per element, kNone = none
  uint8_t* del;
  uint8_t* bad;
  uint32_t maxn, maxe;
};

// Words CTA 0 writes in a scan superstep and every CTA reads after the
// next barrier, so the loop state (node and element counts, worklist size)
// advances identically in every CTA's registers.
enum : int { kTotNode = 0, kTotEl, kTotWl, kTotBad, kErr, kStateWords };
enum : uint32_t { kErrCapacity = 1, kErrCavity = 2, kErrRounds = 3, kErrMesh = 4 };

struct DmrWs {
  uint32_t* wl[2];            // worklists, capacity maxe each
  unsigned long long* own;    // per element: (~stamp << 32) | item
  uint32_t* cav;              // chunk x kCav
  uint32_t* bnd;              // chunk x kBnd
  uint32_t* nc;               // per item: cavity elements (0 = inactive)
  uint32_t* bc;               // per item: boundary words
  uint8_t* win;               // per item: commits
  double* cx;
  double* cy;
  uint32_t* c_node;           // per item: nodes, elements, worklist entries -> offsets
  uint32_t* c_el;
  uint32_t* c_wl;
  uint32_t* cta_cnt;          // per CTA: bad new elements -> offsets
  uint32_t* st;               // kStateWords
  uint32_t* out;              // [0] nodes, [1] elements, [2] rounds, [3] chunks, [4] refinements
  uint32_t chunk;
};

// ------------------------------------------------------------- geometry

__device__ __forceinline__ bool seg_of(const uint32_t* e) { return e[2] == kNone; }

__device__ __forceinline__ double sqdist(double ax, double ay, double bx, double by) {
  const double dx = ax - bx;
  const double dy = ay - by;
  return dx * dx + dy * dy;
}

// angle at c below 30 degrees (angleLT, dmr_common.cl:119-142)
__device__ bool small_angle(const DmrMesh& m, uint32_t a, uint32_t b, uint32_t c) {
  const double xa = __ldcg(&m.x[a]), ya = __ldcg(&m.y[a]);
  const double xb = __ldcg(&m.x[b]), yb = __ldcg(&m.y[b]);
  const double xc = __ldcg(&m.x[c]), yc = __ldcg(&m.y[c]);
  const double vax = xa - xc, vay = ya - yc, vbx = xb - xc, vby = yb - yc;
  const double dp = vax * vbx + vay * vby;
  if (dp < 0.0) return false;
  const double da = sqdist(xa, ya, xc, yc);
  const double db = sqdist(xb, yb, xc, yc);
  const double cosv = dp * (1.0 / sqrt(da * db));
  return cosv > 0x1.bb67ae8584cabp-1;  // cos(30 degrees), correctly rounded
}

// angle at c obtuse (angleOB, dmr_common.cl:189-199)
__device__ bool obtuse(const DmrMesh& m, uint32_t a, uint32_t b, uint32_t c) {
  const double xc = __ldcg(&m.x[c]), yc = __ldcg(&m.y[c]);
  const double vax = __ldcg(&m.x[a]) - xc, vay = __ldcg(&m.y[a]) - yc;
  const double vbx = __ldcg(&m.x[b]) - xc, vby = __ldcg(&m.y[b]) - yc;
  return vax * vbx + vay * vby < 0.0;
}

__device__ void load3(const uint32_t* p, uint32_t* o) {
  o[0] = __ldcg(p);
  o[1] = __ldcg(p + 1);
  o[2] = __ldcg(p + 2);
}

__device__ bool triangle_bad(const DmrMesh& m, const uint32_t* e) {
  return small_angle(m, e[0], e[1], e[2]) || small_angle(m, e[2], e[0], e[1]) ||
         small_angle(m, e[1], e[2], e[0]);
}

__device__ __forceinline__ bool holds(const uint32_t* e, uint32_t n) {
  return e[0] == n || e[1] == n || e[2] == n;
}

// the nodes e1 shares with e2, unset ones kNone (find_shared_edge, dmr_common.cl:201-212)
__device__ void common_edge(const uint32_t* e1, const uint32_t* e2, uint32_t* se) {
  int k = 0;
  se[0] = se[1] = kNone;
  if (holds(e2, e1[0])) se[k++] = e1[0];
  if (holds(e2, e1[1])) se[k++] = e1[1];
  if (!seg_of(e1) && holds(e2, e1[2]) && k < 2) se[k++] = e1[2];
}

// the element a bad triangle hands its refinement to: the neighbour across
// the edge facing an obtuse corner, else itself (opposite, dmr_common.cl:214-256)
__device__ uint32_t hand_off(const DmrMesh& m, uint32_t t) {
  uint32_t e[3];
  load3(m.el + 3 * (size_t)t, e);
  if (seg_of(e)) return t;
  uint32_t corner;
  if (obtuse(m, e[0], e[1], e[2])) corner = e[2];
  else if (obtuse(m, e[2], e[0], e[1])) corner = e[1];
  else if (obtuse(m, e[1], e[2], e[0])) corner = e[0];
  else return t;
  uint32_t nb[3], se[2];
  load3(m.nb + 3 * (size_t)t, nb);
  // a triangle of a valid mesh has three neighbours; a missing one counts
  // as sharing no edge (and the caller rejects a kNone hand-off)
  auto faces_corner = [&](uint32_t n) {
    if (n == kNone) return false;
    uint32_t o[3];
    load3(m.el + 3 * (size_t)n, o);
    common_edge(e, o, se);
    return se[0] == corner || se[1] == corner;
  };
  uint32_t pick = nb[0];
  if (faces_corner(nb[0])) {
    pick = nb[1];
    if (faces_corner(nb[1])) pick = nb[2];
  }
  return pick;
}

__device__ void circumcentre(double ax, double ay, double bx, double by, double cx, double cy, double* ox,
                             double* oy) {
  // dmr_common.cl:258-276
  const double d = 2 * (ax * (by - cy) + bx * (cy - ay) + cx * (ay - by));
  *ox = ((ax * ax + ay * ay) * (by - cy) + (bx * bx + by * by) * (cy - ay) + (cx * cx + cy * cy) * (ay - by)) / d;
  *oy = ((ax * ax + ay * ay) * (cx - bx) + (bx * bx + by * by) * (ax - cx) + (cx * cx + cy * cy) * (bx - ax)) / d;
}

__device__ __forceinline__ double orient(double pax, double pay, double pbx, double pby, double pcx, double pcy) {
  const double l = (pax - pcx) * (pby - pcy);  // dmr_common.cl:278-287
  const double r = (pay - pcy) * (pbx - pcx);
  return l - r;
}

__device__ double in_circle(double ax, double ay, double bx, double by, double cx, double cy, double px,
                            double py) {
  // gincircle, dmr_common.cl:290-320
  const double apx = ax - px, bpx = bx - px, cpx = cx - px;
  const double apy = ay - py, bpy = by - py, cpy = cy - py;
  const double bpxcpy = bpx * cpy, cpxbpy = cpx * bpy;
  const double alift = apx * apx + apy * apy;
  const double cpxapy = cpx * apy, apxcpy = apx * cpy;
  const double blift = bpx * bpx + bpy * bpy;
  const double apxbpy = apx * bpy, bpxapy = bpx * apy;
  const double clift = cpx * cpx + cpy * cpy;
  return alift * (bpxcpy - cpxbpy) + blift * (cpxapy - apxcpy) + clift * (apxbpy - bpxapy);
}

// does the new point (px, py) lie in t's circumcircle (triangle) or
// diametral circle (segment) (encroached, dmr_common.cl:322-356)
__device__ bool encroaches(const DmrMesh& m, uint32_t t, const uint32_t* root, double px, double py,
                           bool* is_segment) {
  if (t == kNone) return false;
  uint32_t e[3];
  load3(m.el + 3 * (size_t)t, e);
  const double x0 = __ldcg(&m.x[e[0]]), y0 = __ldcg(&m.y[e[0]]);
  const double x1 = __ldcg(&m.x[e[1]]), y1 = __ldcg(&m.y[e[1]]);
  if (seg_of(e)) {
    *is_segment = true;
    const uint32_t off = root[0] == e[0] ? (root[1] == e[1] ? root[2] : root[1]) : root[0];
    if ((orient(x0, y0, x1, y1, __ldcg(&m.x[off]), __ldcg(&m.y[off])) > 0.0) !=
        (orient(x0, y0, x1, y1, px, py) > 0.0))
      return true;
    const double mx = (x0 + x1) / 2;
    const double my = (y0 + y1) / 2;
    const double r2 = sqdist(mx, my, x0, y0);
    return sqdist(px, py, mx, my) < r2;
  }
  return in_circle(x0, y0, x1, y1, __ldcg(&m.x[e[2]]), __ldcg(&m.y[e[2]]), px, py) > 0.0;
}

// An item's cavity in its own slot of the workspace.
struct Cav {
  uint32_t* cav;
  uint32_t* bnd;
  uint32_t nc, bc;
  double cx, cy;
};

__device__ int cav_put(Cav& k, uint32_t t) {
  for (uint32_t i = 0; i < k.nc; ++i)
    if (k.cav[i] == t) return 0;
  if (k.nc >= kCav) return -1;
  k.cav[k.nc++] = t;
  return 0;
}

__device__ int bnd_put(Cav& k, uint32_t s1, uint32_t s2, uint32_t src, uint32_t dst) {
  for (uint32_t i = 0; i < k.bc; i += 4)
    if ((s1 == k.bnd[i] && s2 == k.bnd[i + 1]) || (s1 == k.bnd[i + 1] && s2 == k.bnd[i])) return 0;
  if (k.bc + 4 > kBnd) return -1;
  k.bnd[k.bc++] = s1;
  k.bnd[k.bc++] = s2;
  k.bnd[k.bc++] = src;
  k.bnd[k.bc++] = dst;
  return 0;
}

// build_cavity (dmr_common.cl:390-446): 1 built, 0 restarted from the
// encroached segment now in cav[0], -1 out of capacity
__device__ int grow_cavity(const DmrMesh& m, Cav& k) {
  uint32_t root[3];
  load3(m.el + 3 * (size_t)k.cav[0], root);
  if (seg_of(root)) {
    k.cx = (__ldcg(&m.x[root[0]]) + __ldcg(&m.x[root[1]])) / 2;
    k.cy = (__ldcg(&m.y[root[0]]) + __ldcg(&m.y[root[1]])) / 2;
  } else {
    circumcentre(__ldcg(&m.x[root[0]]), __ldcg(&m.y[root[0]]), __ldcg(&m.x[root[1]]), __ldcg(&m.y[root[1]]),
                 __ldcg(&m.x[root[2]]), __ldcg(&m.y[root[2]]), &k.cx, &k.cy);
  }
  for (uint32_t ce = 0; ce < k.nc; ++ce) {
    uint32_t nbs[3], here[3];
    load3(m.nb + 3 * (size_t)k.cav[ce], nbs);
    for (int i = 0; i < 3; ++i) {
      const uint32_t n = nbs[i];
      if (n == k.cav[0] || n == kNone) continue;
      bool sg = false;
      uint32_t en[3];
      load3(m.el + 3 * (size_t)n, en);
      if (!(seg_of(root) && seg_of(en)) && encroaches(m, n, root, k.cx, k.cy, &sg)) {
        if (!sg) {
          if (cav_put(k, n)) return -1;
        } else {
          k.cav[0] = n;
          k.nc = 1;
          k.bc = 0;
          return 0;
        }
      } else {
        uint32_t se[2];
        load3(m.el + 3 * (size_t)k.cav[ce], here);
        common_edge(here, en, se);
        if (bnd_put(k, se[0], se[1], n, k.cav[ce])) return -1;
      }
    }
  }
  return 1;
}

__device__ void link(uint32_t* nb, uint32_t t) {
  // addneighbour, dmr_common.cl:527-534
  if (nb[0] == t || nb[1] == t || nb[2] == t) return;
  if (nb[0] == kNone) { nb[0] = t; return; }
  if (nb[1] == kNone) { nb[1] = t; return; }
  if (nb[2] == kNone) nb[2] = t;
}

__device__ bool share_edge(const uint32_t* e1, const uint32_t* e2) {
  // adjacent, dmr_common.cl:510-525
  int k = (int)holds(e2, e1[0]) + (int)holds(e2, e1[1]);
  if (!seg_of(e1)) k += (int)holds(e2, e1[2]);
  return k == 2;
}

__device__ void new_triangle(const DmrMesh& m, uint32_t n1, uint32_t n2, uint32_t n3, uint32_t outside,
                             uint32_t oldt, uint32_t ndx) {
  // add_triangle, dmr_common.cl:475-508
  uint32_t* e = m.el + 3 * (size_t)ndx;
  if (orient(__ldcg(&m.x[n1]), __ldcg(&m.y[n1]), __ldcg(&m.x[n2]), __ldcg(&m.y[n2]), __ldcg(&m.x[n3]),
             __ldcg(&m.y[n3])) > 0) {
    e[0] = n1; e[1] = n2; e[2] = n3;
  } else {
    e[0] = n3; e[1] = n2; e[2] = n1;
  }
  m.bad[ndx] = 0;
  m.del[ndx] = 0;
  uint32_t* nb = m.nb + 3 * (size_t)ndx;
  nb[0] = outside;
  nb[1] = nb[2] = kNone;
  uint32_t* o = m.nb + 3 * (size_t)outside;  // owned by this item
  if (__ldcg(&o[0]) == oldt) o[0] = ndx;
  else if (__ldcg(&o[1]) == oldt) o[1] = ndx;
  else o[2] = ndx;
}

__device__ void new_segment(const DmrMesh& m, uint32_t n1, uint32_t n2, uint32_t ndx) {
  // add_segment, dmr_common.cl:462-473
  uint32_t* e = m.el + 3 * (size_t)ndx;
  e[0] = n1; e[1] = n2; e[2] = kNone;
  m.bad[ndx] = 0;
  m.del[ndx] = 0;
  uint32_t* nb = m.nb + 3 * (size_t)ndx;
  nb[0] = nb[1] = nb[2] = kNone;
}

// ------------------------------------------------------------- scans

// Exclusive prefix sum of a[0, n) in place by every thread of one CTA;
// returns the total.
__device__ uint32_t cta_scan(uint32_t* a, uint32_t n) {
  __shared__ uint32_t warp_tot[kBlock / 32];
  __shared__ uint32_t carry;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint32_t base = 0; base < n; base += blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = i < n ? a[i] : 0u;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
      uint32_t t = lane < nw ? warp_tot[lane] : 0u;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, t, o);
        if (lane >= o) t += y;
      }
      if (lane < nw) warp_tot[lane] = t;
    }
    __syncthreads();
    const uint32_t before = carry + (w ? warp_tot[w - 1] : 0u) + x - v;
    if (i < n) a[i] = before;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = before + v;
    __syncthreads();
  }
  return carry;
}

__device__ __forceinline__ unsigned long long own_key(uint32_t stamp, uint32_t item) {
  return ((unsigned long long)(0xFFFFFFFFu - stamp) << 32) | item;
}

// i-th element item t claimed: its cavity elements, then the outside
// neighbour of every boundary record
__device__ __forceinline__ uint32_t claim_of(const DmrWs& ws, uint32_t t, uint32_t i, uint32_t nc) {
  return i < nc ? ws.cav[(size_t)t * kCav + i] : ws.bnd[(size_t)t * kBnd + 4 * (i - nc) + 2];
}

__device__ __forceinline__ void raise_dmr(const DmrWs& ws, uint32_t code) { atomicCAS(&ws.st[kErr], 0u, code); }

// is element t a live triangle that is (or now tests) bad
__device__ bool live_bad(const DmrMesh& m, uint32_t t, bool test) {
  uint32_t e[3];
  load3(m.el + 3 * (size_t)t, e);
  if (seg_of(e) || __ldcg(&m.del[t])) return false;
  if (__ldcg(&m.bad[t])) return true;
  if (!test) return false;
  const bool b = triangle_bad(m, e);
  if (b) m.bad[t] = 1;
  return b;
}

// ------------------------------------------------------------- kernel

// Bad triangles among elements [from, to) appended to `out` after `base`
// entries in element order (check_triangles, dmr_common.cl:144-187): every
// CTA tests a contiguous share, CTA 0 scans the per-CTA counts, every CTA
// appends its share at its offset.  Returns the entries appended (the same
// in every CTA), or ~0u when a barrier failed.
template <class Sync>
__device__ uint32_t check_new(Sync& s, const DmrMesh& m, const DmrWs& ws, uint32_t from, uint32_t to,
                              uint32_t* out, uint32_t base) {
  const uint32_t P = (uint32_t)s.P(), id = (uint32_t)s.id();
  const uint32_t n = to > from ? to - from : 0;
  const uint32_t per = (n + P - 1) / P;
  const uint32_t lo = from + min(n, id * per), hi = from + min(n, (id + 1) * per);
  uint32_t mine = 0;
  for (uint32_t t = lo + threadIdx.x; t < hi; t += blockDim.x) mine += live_bad(m, t, true);
  mine = __reduce_add_sync(kFull, mine);
  __shared__ uint32_t part[kBlock / 32];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = mine;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t tot = 0;
    for (uint32_t w = 0; w < blockDim.x / 32; ++w) tot += part[w];
    ws.cta_cnt[id] = tot;
  }
  if (!s.sync()) return ~0u;
  if (id == 0) {
    const uint32_t tot = cta_scan(ws.cta_cnt, P);
    if (threadIdx.x == 0) ws.st[kTotBad] = tot;
  }
  if (!s.sync()) return ~0u;
  if (threadIdx.x == 0) {
    uint32_t at = base + __ldcg(&ws.cta_cnt[id]);
    for (uint32_t t = lo; t < hi; ++t)
      if (live_bad(m, t, false)) out[at++] = t;
  }
  const uint32_t added = (uint32_t)cta_words<1>([&](unsigned long long* w) { w[0] = __ldcg(&ws.st[kTotBad]); })[0];
  if (!s.sync()) return ~0u;
  return added;
}

template <class Sync>
__device__ void dmr_body(Sync& s, const DmrMesh& m, const DmrWs& ws, uint32_t nnodes0, uint32_t nelements0) {
  const Warps W = warps_of(s.id(), s.P());
  const bool leader = s.id() == 0 && threadIdx.x == 0;
  // loop state, identical in every CTA
  uint32_t nn = nnodes0, ne = nelements0, parity = 0, rounds = 0, steps = 0, refined = 0;
  uint32_t nw = check_new(s, m, ws, 0, ne, ws.wl[0], 0);
  if (nw == ~0u) return;
  uint32_t err = 0;
  while (nw && !err) {
    if (++rounds > kMaxRounds) {
      err = kErrRounds;
      break;
    }
    const uint32_t last = ne;
    const uint32_t* wl = ws.wl[parity];
    uint32_t* nwl = ws.wl[parity ^ 1];
    uint32_t nwl_n = 0;
    for (uint32_t s0 = 0; s0 < nw; s0 += ws.chunk) {
      const uint32_t cnt = min(ws.chunk, nw - s0);
      const uint32_t stamp = ++steps;
      // -- build every item's cavity from the mesh as the chunk found it
      //    (dmr_port_kernel.cl:58-85) and claim it: the lowest item wins
      for (uint32_t t = W.gthread; t < cnt; t += W.nthreads) {
        const uint32_t ele = __ldcg(&wl[s0 + t]);
        ws.nc[t] = 0;
        if (!(ele < last && __ldcg(&m.bad[ele]) && !__ldcg(&m.del[ele]))) continue;
        Cav k{ws.cav + (size_t)t * kCav, ws.bnd + (size_t)t * kBnd, 1, 0, 0.0, 0.0};
        k.cav[0] = hand_off(m, ele);
        if (k.cav[0] == kNone) {
          raise_dmr(ws, kErrMesh);
          continue;
        }
        int r = grow_cavity(m, k);
        if (r == 0) r = grow_cavity(m, k);
        if (r < 0) {
          raise_dmr(ws, kErrCavity);
          continue;
        }
        ws.nc[t] = k.nc;
        ws.bc[t] = k.bc;
        ws.cx[t] = k.cx;
        ws.cy[t] = k.cy;
        const unsigned long long key = own_key(stamp, t);
        for (uint32_t i = 0; i < k.nc + k.bc / 4; ++i) atomicMin(&ws.own[claim_of(ws, t, i, k.nc)], key);
      }
      if (!s.sync()) return;
      // -- ownership test (dmr_port_kernel.cl:90-129) and slot counts
      for (uint32_t t = W.gthread; t < cnt; t += W.nthreads) {
        const uint32_t nc = ws.nc[t];
        uint32_t cn = 0, ce = 0, cw = 0;
        bool w = false;
        if (nc) {
          const uint32_t nbd = ws.bc[t] / 4;
          const unsigned long long key = own_key(stamp, t);
          w = true;
          for (uint32_t i = 0; i < nc + nbd && w; ++i) w = __ldcg(&ws.own[claim_of(ws, t, i, nc)]) == key;
          if (w) {
            uint32_t root[3];
            load3(m.el + 3 * (size_t)ws.cav[(size_t)t * kCav], root);
            cn = 1;
            ce = nbd + (seg_of(root) ? 2u : 0u);
            const uint32_t ele = __ldcg(&wl[s0 + t]);
            cw = 1;
            for (uint32_t i = 0; i < nc; ++i)
              if (ws.cav[(size_t)t * kCav + i] == ele) cw = 0;  // the bad triangle itself went: no repush
          } else {
            cw = 1;  // lost a claim: back on the worklist
          }
        }
        ws.win[t] = w;
        ws.c_node[t] = cn;
        ws.c_el[t] = ce;
        ws.c_wl[t] = cw;
      }
      if (!s.sync()) return;
      // -- slots in item order (the reference's atomic_add, dmr_port_kernel.cl:137-141)
      if (s.id() == 0) {
        const uint32_t tn = cta_scan(ws.c_node, cnt);
        const uint32_t te = cta_scan(ws.c_el, cnt);
        const uint32_t tw = cta_scan(ws.c_wl, cnt);
        if (threadIdx.x == 0) {
          ws.st[kTotNode] = tn;
          ws.st[kTotEl] = te;
          ws.st[kTotWl] = tw;
          if (nn + tn > m.maxn || ne + te > m.maxe) raise_dmr(ws, kErrCapacity);
        }
      }
      if (!s.sync()) return;
      const unsigned long long* tot = cta_words<4>([&](unsigned long long* w) {
        w[0] = __ldcg(&ws.st[kTotNode]);
        w[1] = __ldcg(&ws.st[kTotEl]);
        w[2] = __ldcg(&ws.st[kTotWl]);
        w[3] = __ldcg(&ws.st[kErr]);
      });
      const uint32_t tn = (uint32_t)tot[0], te = (uint32_t)tot[1], tw = (uint32_t)tot[2];
      err = (uint32_t)tot[3];
      if (err) break;
      // -- commit (dmr_port_kernel.cl:130-186): every write lands in a new
      //    slot or in an element the item owns
      for (uint32_t t = W.gthread; t < cnt; t += W.nthreads) {
        const uint32_t nc = ws.nc[t];
        if (!nc) continue;
        const uint32_t ele = __ldcg(&wl[s0 + t]);
        if (!ws.win[t]) {
          nwl[nwl_n + ws.c_wl[t]] = ele;
          continue;
        }
        const uint32_t* cav = ws.cav + (size_t)t * kCav;
        const uint32_t* bnd = ws.bnd + (size_t)t * kBnd;
        const uint32_t bc = ws.bc[t];
        uint32_t root[3];
        load3(m.el + 3 * (size_t)cav[0], root);
        const uint32_t cnode = nn + ws.c_node[t];
        m.x[cnode] = ws.cx[t];
        m.y[cnode] = ws.cy[t];
        const uint32_t first = ne + ws.c_el[t];
        uint32_t nx = first;
        if (seg_of(root)) {
          new_segment(m, root[0], cnode, nx++);
          new_segment(m, cnode, root[1], nx++);
        }
        for (uint32_t i = 0; i < bc; i += 4) new_triangle(m, bnd[i], bnd[i + 1], cnode, bnd[i + 2], bnd[i + 3], nx++);
        // setup_neighbours among the new elements (dmr_common.cl:538-555)
        for (uint32_t i = first; i < nx; ++i)
          for (uint32_t j = i + 1; j < nx; ++j) {
            uint32_t ei[3], ej[3];
            load3(m.el + 3 * (size_t)i, ei);
            load3(m.el + 3 * (size_t)j, ej);
            if (share_edge(ei, ej)) {
              link(m.nb + 3 * (size_t)i, j);
              link(m.nb + 3 * (size_t)j, i);
            }
          }
        bool repush = true;
        for (uint32_t i = 0; i < nc; ++i) {
          m.del[cav[i]] = 1;
          if (cav[i] == ele) repush = false;
        }
        if (repush) nwl[nwl_n + ws.c_wl[t]] = ele;
      }
      nn += tn;
      ne += te;
      nwl_n += tw;
      refined += tn;
      if (!s.sync()) return;
    }
    if (err) break;
    // -- the bad triangles among this round's new elements, in element order
    const uint32_t added = check_new(s, m, ws, last, ne, nwl, nwl_n);
    if (added == ~0u) return;
    nw = nwl_n + added;
    parity ^= 1;
  }
  if (leader) {
    ws.out[0] = nn;
    ws.out[1] = ne;
    ws.out[2] = rounds;
    ws.out[3] = steps;
    ws.out[4] = refined;
    if (err) atomicCAS(&ws.st[kErr], 0u, err);
  }
}

__global__ void __launch_bounds__(kBlock) k_dmr_xf(DiscoveryArgs a, DmrMesh m, DmrWs ws, uint32_t nnodes0,
                                                   uint32_t nelements0) {
  __shared__ LocalCtx l;
  if (!discover(a, &l)) return;
  XfSync s{&a, &l};
  dmr_body(s, m, ws, nnodes0, nelements0);
}

}  // namespace

using namespace gdbi;

// find_neighbours_cpu (lonestar_gpu_opencl/apps/dmr/dmr.h:55-104): elements in
// index order, each edge of a triangle (one of a segment) keyed by its
// sorted node pair; an edge seen a second time links the two elements, in
// the order the reference's map links them.
static void mesh_neighbours(uint32_t ne, const uint32_t* el, uint32_t* nb) {
  std::unordered_map<uint64_t, uint32_t> open;
  open.reserve(2 * (size_t)ne);
  auto add = [](uint32_t* n, uint32_t t) {
    if (n[0] == t || n[1] == t || n[2] == t) return;
    if (n[0] == kNone) n[0] = t;
    else if (n[1] == kNone) n[1] = t;
    else if (n[2] == kNone) n[2] = t;
  };
  for (uint32_t t = 0; t < ne; ++t) {
    uint32_t* n = nb + 3 * (size_t)t;
    n[0] = n[1] = n[2] = kNone;
  }
  for (uint32_t t = 0; t < ne; ++t) {
    uint32_t v[3] = {el[3 * (size_t)t], el[3 * (size_t)t + 1], el[3 * (size_t)t + 2]};
    std::sort(v, v + 3);
    const uint64_t edges[3] = {((uint64_t)v[0] << 32) | v[1], ((uint64_t)v[1] << 32) | v[2],
                               ((uint64_t)v[0] << 32) | v[2]};
    const int count = el[3 * (size_t)t + 2] == kNone ? 1 : 3;
    for (int i = 0; i < count; ++i) {
      auto it = open.find(edges[i]);
      if (it != open.end()) {
        add(nb + 3 * (size_t)it->second, t);
        add(nb + 3 * (size_t)t, it->second);
        open.erase(it);
      } else {
        open.emplace(edges[i], t);
      }
    }
  }
}

extern "C" int gdb_dmr_refine(gdb_ctx* c, const double* x, const double* y, uint32_t nnodes,
                              const uint32_t* elements, uint32_t nelements, uint32_t maxfactor,
                              uint32_t chunk, double* x_out, double* y_out, uint32_t* el_out,
                              uint32_t* nb_out, uint8_t* isdel_out, uint32_t* counts) {
  if (!c || !x || !y || !elements || !x_out || !y_out || !el_out || !nb_out || !isdel_out || !counts ||
      nnodes == 0 || nelements == 0 || maxfactor < 2 || chunk == 0 || chunk > GDB_DMR_MAX_CHUNK)
    return GDB_ERR_INVALID;
  const uint64_t maxn64 = (uint64_t)(maxfactor / 2) * nnodes, maxe64 = (uint64_t)maxfactor * nelements;
  if (maxn64 >= kNone || maxe64 >= kNone) return set_error(c, GDB_ERR_INVALID, "mesh capacity too large");
  const uint32_t maxn = (uint32_t)maxn64, maxe = (uint32_t)maxe64;
  // every node id in range: a segment's third node is the INVALIDID marker
  for (uint64_t i = 0; i < 3ull * nelements; ++i) {
    const uint32_t v = elements[i];
    if (v >= nnodes && !(i % 3 == 2 && v == kNone))
      return set_error(c, GDB_ERR_INVALID, "element node out of range");
  }
  std::vector<uint32_t> nb((size_t)3 * nelements);
  mesh_neighbours(nelements, elements, nb.data());
  const uint32_t items = std::min(chunk, maxe);
  Shape s;
  int rc = persistent_shape(c, (const void*)k_dmr_xf, kBlock, 0, &s, c->opt.barrier == GDB_BARRIER_XF);
  if (rc) return rc;
  Bump b;
  const size_t o_x = b.take((size_t)maxn * 8), o_y = b.take((size_t)maxn * 8);
  const size_t o_el = b.take((size_t)maxe * 12), o_nb = b.take((size_t)maxe * 12);
  const size_t o_del = b.take(maxe), o_bad = b.take(maxe);
  const size_t o_wl0 = b.take((size_t)maxe * 4), o_wl1 = b.take((size_t)maxe * 4);
  const size_t o_own = b.take((size_t)maxe * 8);
  const size_t o_cav = b.take((size_t)items * kCav * 4), o_bnd = b.take((size_t)items * kBnd * 4);
  const size_t o_nc = b.take((size_t)items * 4), o_bc = b.take((size_t)items * 4), o_win = b.take(items);
  const size_t o_cx = b.take((size_t)items * 8), o_cy = b.take((size_t)items * 8);
  const size_t o_cn = b.take((size_t)items * 4), o_ce = b.take((size_t)items * 4), o_cw = b.take((size_t)items * 4);
  const size_t o_cta = b.take((size_t)std::max(s.grid, 1) * 4);
  const size_t o_st = b.take(128), o_out = b.take(64);
  char* base = (char*)workspace(c, b.off);
  if (!base) return GDB_ERR_OOM;
  DmrMesh m;
  m.x = (double*)(base + o_x);
  m.y = (double*)(base + o_y);
  m.el = (uint32_t*)(base + o_el);
  m.nb = (uint32_t*)(base + o_nb);
  m.del = (uint8_t*)(base + o_del);
  m.bad = (uint8_t*)(base + o_bad);
  m.maxn = maxn;
  m.maxe = maxe;
  DmrWs ws;
  ws.wl[0] = (uint32_t*)(base + o_wl0);
  ws.wl[1] = (uint32_t*)(base + o_wl1);
  ws.own = (unsigned long long*)(base + o_own);
  ws.cav = (uint32_t*)(base + o_cav);
  ws.bnd = (uint32_t*)(base + o_bnd);
  ws.nc = (uint32_t*)(base + o_nc);
  ws.bc = (uint32_t*)(base + o_bc);
  ws.win = (uint8_t*)(base + o_win);
  ws.cx = (double*)(base + o_cx);
  ws.cy = (double*)(base + o_cy);
  ws.c_node = (uint32_t*)(base + o_cn);
  ws.c_el = (uint32_t*)(base + o_ce);
  ws.c_wl = (uint32_t*)(base + o_cw);
  ws.cta_cnt = (uint32_t*)(base + o_cta);
  ws.st = (uint32_t*)(base + o_st);
  ws.out = (uint32_t*)(base + o_out);
  ws.chunk = items;
  cudaStream_t st = c->stream;
  GDB_CUDA(c, cudaMemcpyAsync(m.x, x, (size_t)nnodes * 8, cudaMemcpyHostToDevice, st));
  GDB_CUDA(c, cudaMemcpyAsync(m.y, y, (size_t)nnodes * 8, cudaMemcpyHostToDevice, st));
  GDB_CUDA(c, cudaMemcpyAsync(m.el, elements, (size_t)nelements * 12, cudaMemcpyHostToDevice, st));
  GDB_CUDA(c, cudaMemcpyAsync(m.nb, nb.data(), (size_t)nelements * 12, cudaMemcpyHostToDevice, st));
  GDB_CUDA(c, cudaMemsetAsync(m.del, 0, maxe, st));
  GDB_CUDA(c, cudaMemsetAsync(m.bad, 0, maxe, st));
  GDB_CUDA(c, cudaMemsetAsync(ws.own, 0xFF, (size_t)maxe * 8, st));
  GDB_CUDA(c, cudaMemsetAsync(ws.st, 0, 128, st));
  DiscoveryArgs a = discovery_args(c, s);
  c->last = gdb_run_stats{};
  GDB_CUDA(c, cudaEventRecord(c->ev0, st));
  k_dmr_xf<<<s.grid, kBlock, 0, st>>>(a, m, ws, nnodes, nelements);
  GDB_CUDA(c, cudaGetLastError());
  GDB_CUDA(c, cudaEventRecord(c->ev1, st));
  rc = finish_run(c);
  if (rc) return rc;
  uint32_t h[32];
  GDB_CUDA(c, cudaMemcpy(h, ws.st, 128, cudaMemcpyDeviceToHost));
  if (h[kErr] == kErrCapacity)
    return set_error(c, GDB_ERR_CAPACITY, "mesh refinement ran out of node or element slots (maxfactor)");
  if (h[kErr] == kErrCavity) return set_error(c, GDB_ERR_CAPACITY, "a cavity outgrew its slot");
  if (h[kErr] == kErrRounds) return set_error(c, GDB_ERR_TIMEOUT, "mesh refinement did not finish");
  if (h[kErr] == kErrMesh) return set_error(c, GDB_ERR_INVALID, "a bad triangle without three neighbours");
  GDB_CUDA(c, cudaMemcpy(counts, ws.out, 5 * 4, cudaMemcpyDeviceToHost));
  const uint32_t nn = counts[0], ne = counts[1];
  GDB_CUDA(c, cudaMemcpy(x_out, m.x, (size_t)nn * 8, cudaMemcpyDeviceToHost));
  GDB_CUDA(c, cudaMemcpy(y_out, m.y, (size_t)nn * 8, cudaMemcpyDeviceToHost));
  GDB_CUDA(c, cudaMemcpy(el_out, m.el, (size_t)ne * 12, cudaMemcpyDeviceToHost));
  GDB_CUDA(c, cudaMemcpy(nb_out, m.nb, (size_t)ne * 12, cudaMemcpyDeviceToHost));
  GDB_CUDA(c, cudaMemcpy(isdel_out, m.del, ne, cudaMemcpyDeviceToHost));
  float ms = 0;
  GDB_CUDA(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  int n = 0;
  read_participating(c, &n);
  c->last.participating = n;
  c->last.launched = s.grid;
  c->last.launches = 1;
  c->last.kernel_ms = ms;
  c->last.supersteps = counts[3];
  c->last.work_units = counts[4];
  return GDB_OK;
}
