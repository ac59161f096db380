// Graph file readers for the reference's formats (host code only).
//
//  * Lonestar .gr version 1 (lonestar_gpu_opencl/include/graph.h:143-215,
//    readFromGR): little-endian header of four u64 (version = 1, bytes of
//    edge data, nodes, edges), u64 outIdx[nodes] (end offset of each row),
//    u32 dst[edges], a 4-byte pad when edges is odd, then edges x edge data
//    (u32 weights when the edge-data size is 4).
//  * DIMACS shortest-path text (pannotia/graph_parser/parse.cpp:178-282,
//    parseCOO): "c" comments, "p sp V E", "a u v w" with 1-based ids; in the
//    undirected mode every arc is also added reversed.  Arcs are grouped by
//    source keeping their file order (the reference's stable sort by row).
//  * METIS text (parse.cpp:59-176, parseMetis): "%" comments, a header
//    "V E [fmt]", then one line of 1-based neighbours per vertex (pairs
//    "neighbour weight" when fmt ends in 1).
// The reference builds row pointers only for rows that hold arcs, which
// shifts every later row when a vertex has none; here every vertex gets
// its row (an empty one when it has no arcs).
#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gdb.h"

namespace {

thread_local std::string g_io_err;

int io_error(const std::string& m) {
  g_io_err = m;
  return GDB_ERR_INVALID;
}

struct Arc {
  uint32_t src, dst, w;
};

// Group arcs by source keeping their order (counting sort), into out.
int build_csr(uint64_t V, const std::vector<Arc>& arcs, bool weighted, gdb_csr* out) {
  if (V >= (1ull << 31)) return io_error("more than 2^31 - 1 vertices");
  if (arcs.size() >= (1ull << 32)) return io_error("2^32 or more arcs");
  const uint64_t E = arcs.size();
  uint32_t* row = (uint32_t*)std::malloc((V + 1) * 4);
  uint32_t* col = (uint32_t*)std::malloc(std::max<uint64_t>(E, 1) * 4);
  uint32_t* w = weighted ? (uint32_t*)std::malloc(std::max<uint64_t>(E, 1) * 4) : nullptr;
  if (!row || !col || (weighted && !w)) {
    std::free(row);
    std::free(col);
    std::free(w);
    return GDB_ERR_OOM;
  }
  std::memset(row, 0, (V + 1) * 4);
  for (const Arc& a : arcs) row[a.src + 1]++;
  for (uint64_t v = 0; v < V; ++v) row[v + 1] += row[v];
  std::vector<uint32_t> fill(row, row + V);
  for (const Arc& a : arcs) {
    const uint32_t k = fill[a.src]++;
    col[k] = a.dst;
    if (w) w[k] = a.w;
  }
  out->V = (uint32_t)V;
  out->E = E;
  out->row_ptr = row;
  out->col = col;
  out->w = w;
  return GDB_OK;
}

bool read_file(const char* path, std::string* data) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  data->resize(n > 0 ? (size_t)n : 0);
  const size_t got = n > 0 ? std::fread(&(*data)[0], 1, (size_t)n, f) : 0;
  std::fclose(f);
  return got == data->size();
}

uint64_t le64(const unsigned char* p) {
  uint64_t v = 0;
  for (int i = 7; i >= 0; --i) v = (v << 8) | p[i];
  return v;
}
uint32_t le32(const unsigned char* p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
void put64(std::string& s, uint64_t v) {
  for (int i = 0; i < 8; ++i) s.push_back((char)((v >> (8 * i)) & 0xff));
}
void put32(std::string& s, uint32_t v) {
  for (int i = 0; i < 4; ++i) s.push_back((char)((v >> (8 * i)) & 0xff));
}

int read_gr(const std::string& d, gdb_csr* out) {
  const unsigned char* p = (const unsigned char*)d.data();
  if (d.size() < 32) return io_error(".gr: file shorter than its header");
  const uint64_t version = le64(p), esz = le64(p + 8), V = le64(p + 16), E = le64(p + 24);
  if (version != 1) return io_error(".gr: version is not 1");
  if (esz != 0 && esz != 4) return io_error(".gr: edge data other than 0 or 4 bytes");
  if (V >= (1ull << 31) || E >= (1ull << 32)) return io_error(".gr: graph too large");
  const uint64_t need = 32 + 8 * V + 4 * E + ((E & 1) ? 4 : 0) + esz * E;
  if (d.size() < need) return io_error(".gr: file shorter than its arrays");
  const unsigned char* idx = p + 32;
  const unsigned char* dst = idx + 8 * V;
  const unsigned char* dat = dst + 4 * E + ((E & 1) ? 4 : 0);
  uint32_t* row = (uint32_t*)std::malloc((V + 1) * 4);
  uint32_t* col = (uint32_t*)std::malloc(std::max<uint64_t>(E, 1) * 4);
  uint32_t* w = esz ? (uint32_t*)std::malloc(std::max<uint64_t>(E, 1) * 4) : nullptr;
  if (!row || !col || (esz && !w)) {
    std::free(row);
    std::free(col);
    std::free(w);
    return GDB_ERR_OOM;
  }
  row[0] = 0;
  uint64_t prev = 0;
  int rc = GDB_OK;
  for (uint64_t v = 0; v < V && rc == GDB_OK; ++v) {
    const uint64_t end = le64(idx + 8 * v);
    if (end < prev || end > E) rc = io_error(".gr: row offsets not increasing or past the arcs");
    row[v + 1] = (uint32_t)end;
    prev = end;
  }
  if (rc == GDB_OK && prev != E) rc = io_error(".gr: last row offset differs from the arc count");
  for (uint64_t e = 0; e < E && rc == GDB_OK; ++e) {
    col[e] = le32(dst + 4 * e);
    if (col[e] >= V) rc = io_error(".gr: arc to a vertex out of range");
    if (w) w[e] = le32(dat + 4 * e);
  }
  if (rc != GDB_OK) {
    std::free(row);
    std::free(col);
    std::free(w);
    return rc;
  }
  out->V = (uint32_t)V;
  out->E = E;
  out->row_ptr = row;
  out->col = col;
  out->w = w;
  return GDB_OK;
}

// Next line of text (without the newline); false at the end.
bool next_line(const std::string& d, size_t* pos, std::string* line) {
  if (*pos >= d.size()) return false;
  size_t e = d.find('\n', *pos);
  if (e == std::string::npos) e = d.size();
  line->assign(d, *pos, e - *pos);
  if (!line->empty() && line->back() == '\r') line->pop_back();
  *pos = e + 1;
  return true;
}

int read_dimacs(const std::string& d, bool directed, gdb_csr* out) {
  size_t pos = 0;
  std::string line;
  long long V = -1, Edecl = 0;
  std::vector<Arc> arcs;
  while (next_line(d, &pos, &line)) {
    if (line.empty() || line[0] == 'c') continue;
    if (line[0] == 'p') {
      char kind[16] = {0};
      if (std::sscanf(line.c_str(), "p %15s %lld %lld", kind, &V, &Edecl) != 3 || V < 0 || Edecl < 0)
        return io_error("DIMACS: bad problem line");
      arcs.reserve((size_t)std::min<long long>(Edecl, 1ll << 24) * (directed ? 1 : 2));
    } else if (line[0] == 'a') {
      long long u, v, w;
      if (V < 0) return io_error("DIMACS: arc before the problem line");
      if (std::sscanf(line.c_str(), "a %lld %lld %lld", &u, &v, &w) != 3)
        return io_error("DIMACS: bad arc line");
      if (u < 1 || v < 1 || u > V || v > V) return io_error("DIMACS: vertex id out of range");
      if (w < 0 || w > 0xffffffffll) return io_error("DIMACS: weight out of uint32 range");
      arcs.push_back({(uint32_t)(u - 1), (uint32_t)(v - 1), (uint32_t)w});
      if (!directed) arcs.push_back({(uint32_t)(v - 1), (uint32_t)(u - 1), (uint32_t)w});
    }
  }
  if (V < 0) return io_error("DIMACS: no problem line");
  return build_csr((uint64_t)V, arcs, true, out);
}

int read_metis(const std::string& d, gdb_csr* out) {
  size_t pos = 0;
  std::string line;
  long long V = -1, Edecl = 0;
  bool weighted = false;
  long long v = 0;
  std::vector<Arc> arcs;
  while (next_line(d, &pos, &line)) {
    if (!line.empty() && line[0] == '%') continue;
    if (V < 0) {
      char fmt[16] = {0};
      const int n = std::sscanf(line.c_str(), "%lld %lld %15s", &V, &Edecl, fmt);
      if (n < 2 || V < 0 || Edecl < 0) return io_error("METIS: bad header");
      if (n == 3) {
        const size_t L = std::strlen(fmt);
        if ((L > 1 && fmt[L - 2] == '1') || (L > 2 && fmt[L - 3] == '1'))
          return io_error("METIS: vertex weights and sizes are not supported");
        weighted = fmt[L - 1] == '1';
      }
      arcs.reserve((size_t)std::min<long long>(Edecl, 1ll << 24) * 2);
      continue;
    }
    if (v >= V) {
      // trailing blank lines are allowed, anything else is not
      if (line.find_first_not_of(" \t") != std::string::npos) return io_error("METIS: more lines than vertices");
      continue;
    }
    const char* s = line.c_str();
    char* end = nullptr;
    for (;;) {
      errno = 0;
      const long long t = std::strtoll(s, &end, 10);
      if (end == s) break;
      if (errno || t < 1 || t > V) return io_error("METIS: neighbour id out of range");
      s = end;
      uint32_t w = 0;
      if (weighted) {
        const long long x = std::strtoll(s, &end, 10);
        if (end == s || x < 0 || x > 0xffffffffll) return io_error("METIS: bad edge weight");
        w = (uint32_t)x;
        s = end;
      }
      arcs.push_back({(uint32_t)v, (uint32_t)(t - 1), w});
    }
    ++v;
  }
  if (V < 0) return io_error("METIS: no header");
  if (v < V) return io_error("METIS: fewer lines than vertices");
  return build_csr((uint64_t)V, arcs, weighted, out);
}

bool ends_with(const std::string& s, const char* suf) {
  const size_t n = std::strlen(suf);
  return s.size() >= n && s.compare(s.size() - n, n, suf) == 0;
}

}  // namespace

extern "C" {

const char* gdb_io_last_error(void) { return g_io_err.c_str(); }

int gdb_csr_read(const char* path, int format, int directed, gdb_csr* out) {
  if (!path || !out) return GDB_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  g_io_err.clear();
  const std::string p(path);
  if (format == GDB_FMT_AUTO) {
    if (ends_with(p, ".gr")) format = GDB_FMT_GR;
    else if (ends_with(p, ".graph") || ends_with(p, ".metis")) format = GDB_FMT_METIS;
    else if (ends_with(p, ".dimacs") || ends_with(p, ".txt") || ends_with(p, ".coo")) format = GDB_FMT_DIMACS;
    else return io_error("cannot tell the format from the file name");
  }
  std::string data;
  if (!read_file(path, &data)) return io_error(std::string("cannot read ") + path);
  switch (format) {
    case GDB_FMT_GR: return read_gr(data, out);
    case GDB_FMT_DIMACS: return read_dimacs(data, directed != 0, out);
    case GDB_FMT_METIS: return read_metis(data, out);
    default: return io_error("unknown format");
  }
}

void gdb_csr_free(gdb_csr* csr) {
  if (!csr) return;
  std::free(csr->row_ptr);
  std::free(csr->col);
  std::free(csr->w);
  std::memset(csr, 0, sizeof(*csr));
}

int gdb_csr_write_gr(const char* path, const gdb_csr* c) {
  if (!path || !c || !c->row_ptr || (c->E && !c->col)) return GDB_ERR_INVALID;
  if (c->row_ptr[0] != 0 || c->row_ptr[c->V] != c->E) return io_error(".gr: row_ptr does not span the arcs");
  std::string s;
  s.reserve(32 + 8 * (size_t)c->V + 8 * (size_t)c->E + 4);
  put64(s, 1);
  put64(s, c->w ? 4 : 0);
  put64(s, c->V);
  put64(s, c->E);
  for (uint32_t v = 0; v < c->V; ++v) put64(s, c->row_ptr[v + 1]);
  for (uint64_t e = 0; e < c->E; ++e) put32(s, c->col[e]);
  if (c->E & 1) put32(s, 0);
  if (c->w)
    for (uint64_t e = 0; e < c->E; ++e) put32(s, c->w[e]);
  FILE* f = std::fopen(path, "wb");
  if (!f) return io_error(std::string("cannot write ") + path);
  const bool ok = std::fwrite(s.data(), 1, s.size(), f) == s.size();
  return (std::fclose(f) == 0 && ok) ? GDB_OK : io_error("short write");
}

}  // extern "C"
