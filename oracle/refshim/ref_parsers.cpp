// Test infrastructure: the reference's own Pannotia graph readers
// (pannotia/graph_parser/parse.cpp: parseCOO for DIMACS, parseMetis),
// compiled where they lie and called through a C entry point, to pin the
// library's readers against them.  Output as the reference builds it:
// row pointers only for rows holding arcs (rows = the count of those).
#include "parse.cpp"

extern "C" int ref_parse(const char* path, int metis, int directed, int* nodes, int* edges,
                         int* rows, int** row_array, int** col_array, int** data_array) {
  char buf[4096];
  snprintf(buf, sizeof buf, "%s", path);
  csr_array* c = metis ? parseMetis(buf, nodes, edges, directed != 0)
                       : parseCOO(buf, nodes, edges, directed != 0);
  if (!c) return -1;
  int r = 0;
  while (r < *nodes && c->row_array[r] < *edges) ++r;  // rows with arcs, then the end marker
  *rows = r;
  *row_array = c->row_array;
  *col_array = c->col_array;
  *data_array = c->data_array;
  free(c->col_cnt);
  free(c);
  return 0;
}

extern "C" void ref_parse_free(int* a, int* b, int* c) {
  free(a);
  free(b);
  free(c);
}
