// FP64 drop-in kernels.  Compiled with -fmad=false: the reference (Rust) never fuses
// multiply-adds, so without contraction every expression rounds as it does there.
#define SWK_R double
#define SWK_CARRY false
#define SWK_OPS kOpsFP64
#define SWK_NAME "fp64"
#define SWK_PULL 0
#include "sweep_ops.cuh"

namespace swh {

static int grid_for_cells(int64_t n) {
  int64_t g = (n + 255) / 256;
  if (g < 1) g = 1;
  if (g > 152 * 16) g = 152 * 16;
  return (int)g;
}

cudaError_t launch_update_levels(const DevicePtrs& p, int lowest_allowed, cudaStream_t s) {
  swk::k_update_levels<<<grid_for_cells(p.num_cells), 256, 0, s>>>(
      (uint32_t)p.num_cells, p.change_timescale, p.level, p.timestep_safety, p.max_timestep,
      p.num_levels, lowest_allowed, p.ctl);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  swk::k_level_counts<<<1, 32, 0, s>>>(p.ctl, p.num_levels);
  return cudaGetLastError();
}

cudaError_t launch_level_hist(const DevicePtrs& p, cudaStream_t s) {
  swk::k_level_hist<<<grid_for_cells(p.num_cells), 256, 0, s>>>((uint32_t)p.num_cells, p.level, p.num_levels, p.ctl);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  swk::k_level_counts<<<1, 32, 0, s>>>(p.ctl, p.num_levels);
  return cudaGetLastError();
}

cudaError_t launch_time_series(const DevicePtrs& p, const double* cell_rate, bool carry_neutral, double* partial,
                               double* out6, cudaStream_t s) {
  static_assert(kTimeSeriesPartials == swk::kSeriesBlocks * swk::kSeriesSums, "partial buffer size");
  swk::k_time_series_partial<<<swk::kSeriesBlocks, swk::kSeriesThreads, 0, s>>>(
      (uint32_t)p.num_cells, p.density, p.volume, p.size, p.xhii, carry_neutral ? p.yneu : nullptr, p.temperature,
      cell_rate, partial);
  swk::k_time_series_final<<<1, 32, 0, s>>>(partial, swk::kSeriesBlocks, out6);
  return cudaGetLastError();
}

cudaError_t launch_ionization_time(const DevicePtrs& p, double time, cudaStream_t s, const double* time_dev) {
  swk::k_ionization_time<<<grid_for_cells(p.num_cells), 256, 0, s>>>((uint32_t)p.num_cells, p.xhii,
                                                                     p.ionization_time, time, time_dev);
  return cudaGetLastError();
}

}  // namespace swh
