/* CPU oracle for the discovery-barrier graph path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load this library, and only as the
 * checker (or, in bench.py, as the timed CPU baseline).  The product path
 * (libgdb) never calls it.
 *
 * Each function restates, in plain serial C, the algorithm of one reference
 * kernel; the file:line it follows is given beside it (paths relative to
 * the reference project; pannotia/... = code/experiments/pannotia/...,
 * lonestar/... = code/experiments/lonestar_gpu_opencl/...).
 *
 * Graphs are CSR: row_ptr[V+1], col[E] (0-based, uint32), optional weights
 * w[E].  Parity is pinned against the reference's own OpenCL C kernels,
 * compiled as C++ through oracle/refshim (oracle/_ref), on the fixtures in
 * tests/golden.
 */
#ifndef GDB_ORACLE_H
#define GDB_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Sentinels of the reference. */
#define ORC_LONESTAR_INF 1000000000u /* lonestar/apps/bfs/kernel/bfs_common.cl:35 */
#define ORC_PANNOTIA_BIG 99999999    /* pannotia/graph_app/sssp/kernel/sssp_kernel.cl:68 */

int orc_bfs(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
            uint32_t src, uint32_t* dist);
int orc_sssp_worklist(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
                      const uint32_t* w, uint32_t src, uint32_t* dist);
int orc_sssp_jacobi(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
                    const uint32_t* w, uint32_t src, int32_t* cost,
                    uint32_t* iterations);
int orc_sssp_dijkstra_int(uint32_t V, const uint32_t* row_ptr,
                          const uint32_t* col, const uint32_t* w, uint32_t src,
                          int32_t* cost);
int orc_mis(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
            const float* node_value, int32_t* s_array, uint32_t* rounds);
int orc_color(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
              const float* node_value, int32_t* color, uint32_t* rounds);
int orc_color_fast(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
                   const float* node_value, int32_t* color, uint32_t* rounds);
int orc_bc_f32(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
               const uint32_t* trow, const uint32_t* tcol,
               const uint32_t* sources, uint32_t nsrc, float* bc);
int orc_bc_f64(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
               const uint32_t* sources, uint32_t nsrc, double* bc);
int orc_mst(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
            const uint32_t* w, uint64_t* weight64, uint32_t* weight32,
            uint32_t* components, uint32_t* edges, uint8_t* arc_in_mst);
/* Delaunay mesh refinement (oracle_dmr.c): elements are node triples,
 * segments carry 1234567890 as their third node; outputs sized for
 * (maxfactor / 2) * nnodes nodes and maxfactor * nelements elements;
 * counts = {nodes, elements, rounds, chunks, refinements}. */
int orc_dmr_neighbours(uint32_t ne, const uint32_t* el, uint32_t* nb);
int orc_dmr_refine(const double* x0, const double* y0, uint32_t nnodes,
                   const uint32_t* el0, uint32_t nelements, uint32_t maxfactor,
                   uint32_t chunk, double* x, double* y, uint32_t* el,
                   uint32_t* nb, uint8_t* isdel, uint32_t* counts);
uint32_t orc_dmr_count_bad(const double* x, const double* y, uint32_t ne,
                           const uint32_t* el, const uint8_t* isdel);
uint64_t orc_verify_dist(uint32_t V, const uint32_t* row_ptr,
                         const uint32_t* col, const uint32_t* w,
                         const uint32_t* dist);
uint64_t orc_bfs_reached_arcs(uint32_t V, const uint32_t* row_ptr,
                              const uint32_t* dist, uint32_t inf,
                              uint32_t* reached);

/* Multi-threaded CPU baseline (OpenMP where available): the same phases
 * as the persistent kernels, one parallel loop per barrier interval. */
int orc_par_threads(void);
int orc_par_bfs(uint32_t V, const uint32_t* row_ptr, const uint32_t* col,
                uint32_t src, uint32_t* dist);

#ifdef __cplusplus
}
#endif
#endif
