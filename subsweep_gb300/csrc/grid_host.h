/* Host-side grid producers (Voronoi by half-space clipping, cartesian) that emit the
 * face-neighbour CSR the sweep library consumes.  Workload tooling: not part of the
 * sweep's parity surface. */
#ifndef SUBSWEEP_GRID_HOST_H
#define SUBSWEEP_GRID_HOST_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { SW_HOST_LOCAL = 0, SW_HOST_LOCAL_PERIODIC = 1, SW_HOST_BOUNDARY = 2 };

typedef struct sw_host_grid sw_host_grid;

/* Voronoi tessellation of `n` generators (xyz interleaved) in [0, box)^3. */
sw_host_grid* sw_grid_voronoi(const double* points, int64_t n, const double box_size[3],
                              int32_t periodic, int32_t nthreads);
/* The reference's cartesian test grid (src/sweep/grid/cartesian.rs) on one rank. */
sw_host_grid* sw_grid_cartesian(int32_t nx, int32_t ny, int32_t nz, double cell_size,
                                int32_t periodic);
int64_t sw_grid_num_cells(const sw_host_grid* g);
int64_t sw_grid_num_faces(const sw_host_grid* g);
int64_t sw_grid_failed_cells(const sw_host_grid* g);
int64_t sw_grid_dropped_faces(const sw_host_grid* g);
void sw_grid_copy(const sw_host_grid* g, int64_t* row_ptr, int32_t* nbr, uint8_t* kind,
                  double* area, double* normal, double* volume, double* size, double* position);
void sw_grid_free(sw_host_grid* g);

#ifdef __cplusplus
}
#endif
#endif
