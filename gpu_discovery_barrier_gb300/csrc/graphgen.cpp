// Deterministic synthetic graph generators for the traversal workloads.
//
// Every generator is counter-based (splitmix64 over an index), so the
// graph produced depends only on its parameters and seed -- not on the
// thread count, the host architecture (x86_64 or aarch64) or the order in
// which work is done.  Output is a symmetric CSR with uint32 offsets and
// column ids, rows sorted ascending, no self loops and no duplicate arcs.
//
// The reference reads its inputs from external files (DIMACS road graphs,
// rmat22, grids; pannotia/graph_parser/parse.cpp:178-282,
// lonestar_gpu_opencl/include/graph.h:143-215).  These generators stand in
// for those datasets with the same shapes.

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Hash of an undirected edge {u, v}: identical for both arcs.
inline uint64_t edge_hash(uint64_t seed, uint32_t u, uint32_t v) {
  uint64_t lo = u < v ? u : v, hi = u < v ? v : u;
  return splitmix64(splitmix64(seed) ^ ((lo << 32) | hi));
}

}  // namespace

extern "C" {

uint64_t gdbgen_splitmix64(uint64_t x) { return splitmix64(x); }

// Number of directed arcs of an R x C 4-neighbour grid.
uint64_t gdbgen_grid_arcs(uint32_t R, uint32_t C) {
  return 2ull * ((uint64_t)R * (C - 1) + (uint64_t)C * (R - 1));
}

// R x C 4-neighbour grid; vertex (r, c) has id r*C + c.  Neighbours are
// emitted in ascending id order: up, left, right, down.
int gdbgen_grid(uint32_t R, uint32_t C, uint32_t* row_ptr, uint32_t* col) {
  if (R == 0 || C == 0) return -1;
  uint64_t V = (uint64_t)R * C;
  if (V > 0xFFFFFFFFull || gdbgen_grid_arcs(R, C) > 0xFFFFFFFFull) return -1;
  // Offsets have a closed form, so rows can be filled in parallel.
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < (int64_t)R; ++r) {
    // arcs of all earlier rows: row 0 has no "up" arcs, the others have
    // 2(C-1) horizontal + C up + C down (the last row has no "down" arcs,
    // but it is never an earlier row).
    uint64_t o = 0;
    if (r > 0) {
      const uint64_t row0 = 2ull * (C - 1) + (R > 1 ? C : 0);
      const uint64_t interior = 2ull * (C - 1) + 2ull * C;
      o = row0 + (uint64_t)(r - 1) * interior;
    }
    for (uint32_t c = 0; c < C; ++c) {
      uint64_t id = (uint64_t)r * C + c;
      row_ptr[id] = (uint32_t)o;
      if (r > 0) col[o++] = (uint32_t)(id - C);
      if (c > 0) col[o++] = (uint32_t)(id - 1);
      if (c + 1 < C) col[o++] = (uint32_t)(id + 1);
      if (r + 1 < (int64_t)R) col[o++] = (uint32_t)(id + C);
    }
  }
  row_ptr[V] = (uint32_t)gdbgen_grid_arcs(R, C);
  return 0;
}

// R-MAT: npairs = round(edge_factor * V) generated pairs over [0, V) with
// quadrant probabilities (a, b, c, 1-a-b-c).  Ids are drawn at
// scale = ceil(log2 V) and folded with "% V" when V is not a power of two.
// The result is symmetrised; self loops and duplicates are removed.
// On success *row_ptr_out (V+1) and *col_out (E) are malloc'd; free them
// with gdbgen_free.
int gdbgen_rmat(uint32_t V, double edge_factor, double a, double b, double c,
                uint64_t seed, uint32_t** row_ptr_out, uint32_t** col_out,
                uint64_t* E_out) {
  if (V < 2 || edge_factor <= 0.0) return -1;
  int scale = 0;
  while ((1ull << scale) < V) ++scale;
  const uint64_t npairs = (uint64_t)(edge_factor * (double)V + 0.5);
  const uint64_t tA = (uint64_t)(a * 4294967296.0);
  const uint64_t tB = (uint64_t)((a + b) * 4294967296.0);
  const uint64_t tC = (uint64_t)((a + b + c) * 4294967296.0);

  std::vector<uint32_t> us(npairs), vs(npairs);
  const uint64_t s0 = splitmix64(seed ^ 0x5A17C0DEull);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)npairs; ++i) {
    uint64_t state = s0 ^ ((uint64_t)i * 0xD1B54A32D192ED03ull);
    uint64_t u = 0, v = 0, r = 0;
    for (int l = 0; l < scale; ++l) {
      uint64_t x;
      if ((l & 1) == 0) {
        state = splitmix64(state);
        r = state;
        x = r & 0xFFFFFFFFull;
      } else {
        x = r >> 32;
      }
      uint64_t ub, vb;
      if (x < tA) { ub = 0; vb = 0; }
      else if (x < tB) { ub = 0; vb = 1; }
      else if (x < tC) { ub = 1; vb = 0; }
      else { ub = 1; vb = 1; }
      u = (u << 1) | ub;
      v = (v << 1) | vb;
    }
    us[i] = (uint32_t)(u % V);
    vs[i] = (uint32_t)(v % V);
  }

  // Bucket both arc directions by source.
  std::vector<uint64_t> cnt((size_t)V + 1, 0);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)npairs; ++i) {
    if (us[i] == vs[i]) continue;
    __atomic_fetch_add(&cnt[us[i]], 1ull, __ATOMIC_RELAXED);
    __atomic_fetch_add(&cnt[vs[i]], 1ull, __ATOMIC_RELAXED);
  }
  std::vector<uint64_t> off((size_t)V + 1, 0);
  for (uint32_t i = 0; i < V; ++i) off[i + 1] = off[i] + cnt[i];
  const uint64_t total = off[V];
  std::vector<uint32_t> buf(total);
  std::vector<uint64_t> pos(off.begin(), off.end() - 1);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)npairs; ++i) {
    uint32_t u = us[i], v = vs[i];
    if (u == v) continue;
    buf[__atomic_fetch_add(&pos[u], 1ull, __ATOMIC_RELAXED)] = v;
    buf[__atomic_fetch_add(&pos[v], 1ull, __ATOMIC_RELAXED)] = u;
  }
  us.clear(); us.shrink_to_fit();
  vs.clear(); vs.shrink_to_fit();

  // Sort and dedupe every row (placement order above is not deterministic;
  // the sorted, unique row is).
  std::vector<uint32_t> ndeg(V, 0);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t u = 0; u < (int64_t)V; ++u) {
    uint32_t* s = buf.data() + off[u];
    uint32_t* e = buf.data() + off[u + 1];
    std::sort(s, e);
    ndeg[u] = (uint32_t)(std::unique(s, e) - s);
  }
  uint64_t E = 0;
  for (uint32_t u = 0; u < V; ++u) E += ndeg[u];
  if (E > 0xFFFFFFFFull) return -2;
  uint32_t* rp = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)V + 1));
  uint32_t* cl = (uint32_t*)malloc(sizeof(uint32_t) * (E ? E : 1));
  if (!rp || !cl) { free(rp); free(cl); return -3; }
  rp[0] = 0;
  for (uint32_t u = 0; u < V; ++u) rp[u + 1] = rp[u] + ndeg[u];
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t u = 0; u < (int64_t)V; ++u)
    memcpy(cl + rp[u], buf.data() + off[u], sizeof(uint32_t) * ndeg[u]);
  *row_ptr_out = rp;
  *col_out = cl;
  *E_out = E;
  return 0;
}

void gdbgen_free(void* p) { free(p); }

// Per-arc weights uniform in [lo, hi], one value per undirected edge (both
// arcs of an edge carry the same weight).
void gdbgen_uniform_weights(uint32_t V, const uint32_t* row_ptr,
                            const uint32_t* col, uint64_t seed, uint32_t lo,
                            uint32_t hi, uint32_t* w) {
  const uint64_t span = (uint64_t)hi - lo + 1;
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t u = 0; u < (int64_t)V; ++u)
    for (uint32_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e)
      w[e] = lo + (uint32_t)(edge_hash(seed, (uint32_t)u, col[e]) % span);
}

// Seeded permutation of [0, n) (Fisher-Yates over a splitmix64 stream).
void gdbgen_permutation(uint32_t n, uint64_t seed, uint32_t* out) {
  for (uint32_t i = 0; i < n; ++i) out[i] = i;
  uint64_t s = splitmix64(seed ^ 0xFEEDF00Dull);
  for (uint32_t i = n; i > 1; --i) {
    s = splitmix64(s);
    uint32_t j = (uint32_t)(s % i);
    uint32_t t = out[i - 1];
    out[i - 1] = out[j];
    out[j] = t;
  }
}

// Unique weights: the undirected edges, numbered in CSR order of their
// (u < v) arc, get a seeded permutation of 1..E_undirected; both arcs of an
// edge carry the same weight.  Rows must be sorted (binary search for the
// reverse arc).  Returns the number of undirected edges.
uint64_t gdbgen_unique_weights(uint32_t V, const uint32_t* row_ptr,
                               const uint32_t* col, uint64_t seed,
                               uint32_t* w) {
  // index of each (u<v) arc among the undirected edges
  std::vector<uint64_t> base((size_t)V + 1, 0);
  for (uint32_t u = 0; u < V; ++u) {
    uint64_t k = 0;
    const uint32_t* s = col + row_ptr[u];
    const uint32_t* e = col + row_ptr[u + 1];
    k = (uint64_t)(e - std::upper_bound(s, e, u));
    base[u + 1] = base[u] + k;
  }
  const uint64_t Eu = base[V];
  std::vector<uint32_t> perm(Eu);
  gdbgen_permutation((uint32_t)Eu, seed, perm.data());
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t u = 0; u < (int64_t)V; ++u) {
    const uint32_t* s = col + row_ptr[u];
    const uint32_t* e = col + row_ptr[u + 1];
    const uint32_t* first_up = std::upper_bound(s, e, (uint32_t)u);
    for (const uint32_t* p = s; p < e; ++p) {
      uint32_t v = *p;
      uint64_t idx;
      if (v > (uint32_t)u) {
        idx = base[u] + (uint64_t)(p - first_up);
      } else {
        const uint32_t* vs = col + row_ptr[v];
        const uint32_t* ve = col + row_ptr[v + 1];
        const uint32_t* fu = std::upper_bound(vs, ve, v);
        const uint32_t* q = std::lower_bound(fu, ve, (uint32_t)u);
        idx = base[v] + (uint64_t)(q - fu);
      }
      w[p - col] = perm[idx] + 1;
    }
  }
  return Eu;
}

// `count` distinct seeded sources among the vertices with at least one arc.
// Returns how many were found (fewer only if the graph has fewer such
// vertices).
uint32_t gdbgen_sources(uint32_t V, const uint32_t* row_ptr, uint64_t seed,
                        uint32_t count, uint32_t* out) {
  uint32_t nonisolated = 0;
  for (uint32_t u = 0; u < V; ++u) nonisolated += row_ptr[u + 1] > row_ptr[u];
  if (count > nonisolated) count = nonisolated;
  uint64_t s = splitmix64(seed ^ 0x50C0FFEEull);
  uint32_t got = 0;
  while (got < count) {
    s = splitmix64(s);
    uint32_t v = (uint32_t)(s % V);
    if (row_ptr[v + 1] == row_ptr[v]) continue;
    bool dup = false;
    for (uint32_t k = 0; k < got; ++k) dup |= out[k] == v;
    if (!dup) out[got++] = v;
  }
  return got;
}

// Transpose of a CSR (for the pull-direction kernels); for the symmetric
// graphs generated here it reproduces the input.
void gdbgen_transpose(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
                      const uint32_t* w, uint32_t* trow, uint32_t* tcol,
                      uint32_t* tw) {
  std::vector<uint32_t> cnt((size_t)V + 1, 0);
  for (uint32_t u = 0; u < V; ++u)
    for (uint32_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e) cnt[col[e] + 1]++;
  trow[0] = 0;
  for (uint32_t v = 0; v < V; ++v) trow[v + 1] = trow[v] + cnt[v + 1];
  std::vector<uint32_t> pos(trow, trow + V);
  for (uint32_t u = 0; u < V; ++u)
    for (uint32_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e) {
      uint32_t p = pos[col[e]]++;
      tcol[p] = u;
      if (w && tw) tw[p] = w[e];
    }
}

}  // extern "C"
