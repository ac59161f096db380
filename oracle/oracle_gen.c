/* Workload generator restated for the CPU side -- TEST INFRASTRUCTURE.
 *
 * The timed CPU implementation of the path and the parity checks need the
 * same seeded inputs as the GPU side, without loading any library of the
 * product.  This file restates, in plain C, the counter-based generators the
 * workloads are defined by:
 *
 *   splitmix64(x): x += 0x9E3779B97F4A7C15; then two xor-shift-multiply
 *     rounds (constants 0xBF58476D1CE4E5B9, 0x94D049BB133111EB) and a final
 *     xor-shift by 31 (Steele, Lea, Flood, OOPSLA 2014);
 *   R-MAT (Chakrabarti, Zhan, Faloutsos, SDM 2004): pair i draws its
 *     scale = ceil(log2 V) quadrant choices from the 32-bit halves of the
 *     stream state_i = splitmix64^k(s0 ^ i * 0xD1B54A32D192ED03), s0 =
 *     splitmix64(seed ^ 0x5A17C0DE), low half first; a half x picks quadrant
 *     (0,0) if x < a*2^32, (0,1) if x < (a+b)*2^32, (1,0) if x <
 *     (a+b+c)*2^32, else (1,1); ids fold with "% V"; the pairs are
 *     symmetrised, self loops dropped, rows sorted and deduplicated;
 *   uniform weights: w(u,v) = lo + h(min,max) % (hi-lo+1), h = splitmix64(
 *     splitmix64(seed) ^ (min << 32 | max)), the same on both arcs;
 *   permutation: Fisher-Yates from the top over splitmix64 draws, state
 *     splitmix64(seed ^ 0xFEEDF00D), j = draw % i;
 *   unique weights: undirected edges numbered in CSR order of their u < v
 *     arc receive perm(E_undirected) + 1;
 *   sources: distinct non-isolated vertices drawn as draw % V from state
 *     splitmix64(seed ^ 0x50C0FFEE).
 *
 * tests/test_oracle_gen.py checks every function against the product's
 * generator bit for bit.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

static uint64_t og_mix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

static uint64_t og_edge_hash(uint64_t seed, uint32_t u, uint32_t v) {
  uint64_t lo = u < v ? u : v, hi = u < v ? v : u;
  return og_mix(og_mix(seed) ^ ((lo << 32) | hi));
}

/* insertion sort for short rows, heap sort above 32 entries */
static void og_sift(uint32_t* a, int64_t root, int64_t n) {
  for (;;) {
    int64_t c = 2 * root + 1;
    if (c >= n) return;
    if (c + 1 < n && a[c + 1] > a[c]) ++c;
    if (a[root] >= a[c]) return;
    uint32_t t = a[root]; a[root] = a[c]; a[c] = t;
    root = c;
  }
}

static void og_sort(uint32_t* a, int64_t n) {
  if (n <= 32) {
    for (int64_t i = 1; i < n; ++i) {
      uint32_t x = a[i];
      int64_t j = i - 1;
      while (j >= 0 && a[j] > x) { a[j + 1] = a[j]; --j; }
      a[j + 1] = x;
    }
    return;
  }
  for (int64_t i = n / 2 - 1; i >= 0; --i) og_sift(a, i, n);
  for (int64_t e = n - 1; e > 0; --e) {
    uint32_t t = a[0]; a[0] = a[e]; a[e] = t;
    og_sift(a, 0, e);
  }
}

/* R-MAT pairs -> symmetric sorted unique CSR.  row_ptr and col are
 * malloc'd here (free with orc_gen_free).  0 on success. */
int orc_gen_rmat(uint32_t V, double edge_factor, double a, double b, double c, uint64_t seed,
                 uint32_t** row_ptr_out, uint32_t** col_out, uint64_t* E_out) {
  if (V < 2 || edge_factor <= 0.0) return -1;
  int scale = 0;
  while ((1ull << scale) < V) ++scale;
  const int64_t npairs = (int64_t)(edge_factor * (double)V + 0.5);
  const uint64_t tA = (uint64_t)(a * 4294967296.0);
  const uint64_t tB = (uint64_t)((a + b) * 4294967296.0);
  const uint64_t tC = (uint64_t)((a + b + c) * 4294967296.0);
  const uint64_t s0 = og_mix(seed ^ 0x5A17C0DEull);

  uint32_t* pu = malloc(sizeof(uint32_t) * (size_t)(npairs ? npairs : 1));
  uint32_t* pv = malloc(sizeof(uint32_t) * (size_t)(npairs ? npairs : 1));
  uint64_t* deg = calloc((size_t)V + 1, sizeof(uint64_t));
  if (!pu || !pv || !deg) { free(pu); free(pv); free(deg); return -3; }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < npairs; ++i) {
    uint64_t st = s0 ^ ((uint64_t)i * 0xD1B54A32D192ED03ull), draw = 0, u = 0, v = 0;
    for (int l = 0; l < scale; ++l) {
      uint64_t half;
      if (l % 2 == 0) { st = og_mix(st); draw = st; half = draw & 0xFFFFFFFFull; }
      else half = draw >> 32;
      int qu = half >= tB, qv = (half >= tA && half < tB) || half >= tC;
      u = 2 * u + (uint64_t)qu;
      v = 2 * v + (uint64_t)qv;
    }
    pu[i] = (uint32_t)(u % V);
    pv[i] = (uint32_t)(v % V);
  }
  for (int64_t i = 0; i < npairs; ++i)
    if (pu[i] != pv[i]) { deg[pu[i]]++; deg[pv[i]]++; }
  uint64_t* start = malloc(sizeof(uint64_t) * ((size_t)V + 1));
  if (!start) { free(pu); free(pv); free(deg); return -3; }
  start[0] = 0;
  for (uint32_t x = 0; x < V; ++x) start[x + 1] = start[x] + deg[x];
  uint32_t* arcs = malloc(sizeof(uint32_t) * (size_t)(start[V] ? start[V] : 1));
  if (!arcs) { free(pu); free(pv); free(deg); free(start); return -3; }
  memcpy(deg, start, sizeof(uint64_t) * V); /* deg becomes the fill cursor */
  for (int64_t i = 0; i < npairs; ++i) {
    uint32_t u = pu[i], v = pv[i];
    if (u == v) continue;
    arcs[deg[u]++] = v;
    arcs[deg[v]++] = u;
  }
  free(pu);
  free(pv);
  /* per row: sort, squeeze duplicates to the front, keep the count */
#pragma omp parallel for schedule(dynamic, 512)
  for (int64_t x = 0; x < (int64_t)V; ++x) {
    uint32_t* r = arcs + start[x];
    int64_t n = (int64_t)(start[x + 1] - start[x]), k = 0;
    og_sort(r, n);
    for (int64_t j = 0; j < n; ++j)
      if (k == 0 || r[k - 1] != r[j]) r[k++] = r[j];
    deg[x] = (uint64_t)k;
  }
  uint64_t E = 0;
  for (uint32_t x = 0; x < V; ++x) E += deg[x];
  if (E > 0xFFFFFFFFull) { free(deg); free(start); free(arcs); return -2; }
  uint32_t* rp = malloc(sizeof(uint32_t) * ((size_t)V + 1));
  uint32_t* cl = malloc(sizeof(uint32_t) * (size_t)(E ? E : 1));
  if (!rp || !cl) { free(rp); free(cl); free(deg); free(start); free(arcs); return -3; }
  rp[0] = 0;
  for (uint32_t x = 0; x < V; ++x) rp[x + 1] = rp[x] + (uint32_t)deg[x];
#pragma omp parallel for schedule(dynamic, 512)
  for (int64_t x = 0; x < (int64_t)V; ++x)
    memcpy(cl + rp[x], arcs + start[x], sizeof(uint32_t) * deg[x]);
  free(deg);
  free(start);
  free(arcs);
  *row_ptr_out = rp;
  *col_out = cl;
  *E_out = E;
  return 0;
}

void orc_gen_free(void* p) { free(p); }

void orc_gen_uniform_weights(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
                             uint64_t seed, uint32_t lo, uint32_t hi, uint32_t* w) {
  const uint64_t span = (uint64_t)hi - lo + 1;
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t u = 0; u < (int64_t)V; ++u)
    for (uint32_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e)
      w[e] = lo + (uint32_t)(og_edge_hash(seed, (uint32_t)u, col[e]) % span);
}

void orc_gen_permutation(uint32_t n, uint64_t seed, uint32_t* out) {
  for (uint32_t i = 0; i < n; ++i) out[i] = i;
  uint64_t st = og_mix(seed ^ 0xFEEDF00Dull);
  for (uint32_t i = n; i >= 2; --i) {
    st = og_mix(st);
    uint32_t j = (uint32_t)(st % i), t = out[i - 1];
    out[i - 1] = out[j];
    out[j] = t;
  }
}

/* first index in row [s, e) holding a value > key */
static uint32_t og_after(const uint32_t* col, uint32_t s, uint32_t e, uint32_t key) {
  while (s < e) {
    uint32_t m = s + (e - s) / 2;
    if (col[m] <= key) s = m + 1; else e = m;
  }
  return s;
}

/* first index in row [s, e) holding a value >= key */
static uint32_t og_at(const uint32_t* col, uint32_t s, uint32_t e, uint32_t key) {
  while (s < e) {
    uint32_t m = s + (e - s) / 2;
    if (col[m] < key) s = m + 1; else e = m;
  }
  return s;
}

uint64_t orc_gen_unique_weights(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
                                uint64_t seed, uint32_t* w) {
  uint64_t* up = malloc(sizeof(uint64_t) * ((size_t)V + 1)); /* edges numbered before row u */
  if (!up) return 0;
  up[0] = 0;
  for (uint32_t u = 0; u < V; ++u)
    up[u + 1] = up[u] + (row_ptr[u + 1] - og_after(col, row_ptr[u], row_ptr[u + 1], u));
  const uint64_t Eu = up[V];
  uint32_t* perm = malloc(sizeof(uint32_t) * (size_t)(Eu ? Eu : 1));
  if (!perm) { free(up); return 0; }
  orc_gen_permutation((uint32_t)Eu, seed, perm);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t u = 0; u < (int64_t)V; ++u) {
    uint32_t s = row_ptr[u], e = row_ptr[u + 1];
    uint32_t first = og_after(col, s, e, (uint32_t)u);
    for (uint32_t k = s; k < e; ++k) {
      uint32_t v = col[k];
      uint64_t id;
      if (v > (uint32_t)u) {
        id = up[u] + (k - first);
      } else {
        uint32_t vs = row_ptr[v], ve = row_ptr[v + 1];
        uint32_t vf = og_after(col, vs, ve, v);
        id = up[v] + (og_at(col, vf, ve, (uint32_t)u) - vf);
      }
      w[k] = perm[id] + 1;
    }
  }
  free(perm);
  free(up);
  return Eu;
}

uint32_t orc_gen_sources(uint32_t V, const uint32_t* row_ptr, uint64_t seed, uint32_t count,
                         uint32_t* out) {
  uint32_t live = 0;
  for (uint32_t u = 0; u < V; ++u) live += row_ptr[u + 1] != row_ptr[u];
  if (count > live) count = live;
  uint64_t st = og_mix(seed ^ 0x50C0FFEEull);
  uint32_t got = 0;
  while (got < count) {
    st = og_mix(st);
    uint32_t v = (uint32_t)(st % V);
    if (row_ptr[v + 1] == row_ptr[v]) continue;
    int seen = 0;
    for (uint32_t k = 0; k < got && !seen; ++k) seen = out[k] == v;
    if (!seen) out[got++] = v;
  }
  return got;
}
