/* Voronoi tessellation on the GPU (csrc/voronoi_gpu.cu): the same face-neighbour CSR
 * as the host producer of grid_host.h, built one thread per cell. */
#ifndef SUBSWEEP_VORONOI_GPU_H
#define SUBSWEEP_VORONOI_GPU_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct sw_gpu_grid sw_gpu_grid;

/* Voronoi tessellation of `n` generators (xyz interleaved) in [0, box)^3 on `device`
 * (made the calling thread's current device); null for invalid arguments.
 * sw_gpu_grid_status() is the CUDA error of the construction (0: the arrays are valid). */
sw_gpu_grid* sw_gpu_grid_voronoi(const double* points, int64_t n, const double box_size[3], int32_t periodic,
                                 int32_t device);
int32_t sw_gpu_grid_status(const sw_gpu_grid* g);
int64_t sw_gpu_grid_num_faces(const sw_gpu_grid* g);
int64_t sw_gpu_grid_failed_cells(const sw_gpu_grid* g);
int64_t sw_gpu_grid_dropped_faces(const sw_gpu_grid* g);
void sw_gpu_grid_copy(const sw_gpu_grid* g, int64_t* row_ptr, int32_t* nbr, uint8_t* kind, double* area,
                      double* normal, double* volume, double* size);
void sw_gpu_grid_free(sw_gpu_grid* g);

#ifdef __cplusplus
}
#endif
#endif
