// Launchers of the precision-dependent kernels.  Included once by sweep_fp64.cu
// (R = double, reference-exact neutral fraction) and once by sweep_mixed.cu
// (R = float, carried neutral fraction); each defines SWK_R, SWK_CARRY and SWK_OPS.
#pragma once

#include "launch.h"
#include "sweep_device.cuh"

namespace swh {
namespace {

using R = SWK_R;
constexpr bool kCarry = SWK_CARRY;

swk::SweepArgs<R> sweep_args(const DevicePtrs& p, int level) {
  swk::SweepArgs<R> a;
  a.row_ptr = p.row_ptr;
  a.geo64 = static_cast<const swk::Geo64*>(p.geo64);
  a.geo32 = static_cast<const float4*>(p.geo32);
  a.nbr = p.nbr;
  a.size = p.size;
  a.dir64 = p.dir64;
  a.dir32 = p.dir32;
  a.D = p.D;
  a.Dp = p.Dp;
  a.words = p.words;
  a.guard = p.guard;
  a.level = p.level;
  a.order = p.order;
  a.source = p.source;
  a.att = p.att;
  a.rate_scale = p.rate_scale;
  a.threshold = (R)(p.threshold / p.rate_scale);
  a.incoming = static_cast<R*>(p.incoming);
  a.outgoing = static_cast<R*>(p.outgoing);
  a.periodic = static_cast<R*>(p.periodic);
  a.pending = static_cast<R*>(p.pending);
  a.counters = p.counters;
  a.ready = p.ready;
  a.queued = p.queued;
  a.frontier0 = p.frontier0;
  a.frontier1 = p.frontier1;
  a.ctl = p.ctl;
  a.current_level = level;
  a.timeout_ns = p.timeout_ns;
  a.max_rounds = p.max_rounds;
  return a;
}

int grid_for(int64_t work, int block) {
  int64_t g = (work + block - 1) / block;
  if (g < 1) g = 1;
  if (g > 152 * 16) g = 152 * 16;
  return (int)g;
}

cudaError_t occupancy(int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, swk::k_sweep<R>,
                                                       swk::kWarpsPerBlock * 32, 0);
}

cudaError_t attenuation(const DevicePtrs& p, int level, cudaStream_t s) {
  swk::k_attenuation<kCarry><<<grid_for(p.num_cells, 256), 256, 0, s>>>(
      p.order, p.ctl, level, p.density, p.xhii, p.yneu, p.size, p.att);
  return cudaGetLastError();
}

cudaError_t init_counts(const DevicePtrs& p, int level, uint8_t* debug_counts, cudaStream_t s) {
  swk::SweepArgs<R> a = sweep_args(p, level);
  int blocks = grid_for(p.num_cells * 32, swk::kWarpsPerBlock * 32);
  swk::k_init_counts<R><<<blocks, swk::kWarpsPerBlock * 32, 0, s>>>(a, debug_counts);
  return cudaGetLastError();
}

cudaError_t sweep(const DevicePtrs& p, int level, cudaStream_t s) {
  swk::SweepArgs<R> a = sweep_args(p, level);
  void* args[] = {&a};
  return cudaLaunchCooperativeKernel((const void*)swk::k_sweep<R>, dim3(p.coop_blocks),
                                     dim3(swk::kWarpsPerBlock * 32), args, 0, s);
}

cudaError_t fold_periodic(const DevicePtrs& p, cudaStream_t s) {
  if (p.n_periodic_cells == 0) return cudaSuccess;
  swk::k_fold_periodic<R><<<grid_for((int64_t)p.n_periodic_cells * p.Dp, 256), 256, 0, s>>>(
      static_cast<R*>(p.periodic), static_cast<R*>(p.pending), p.periodic_cells, p.n_periodic_cells, p.Dp);
  return cudaGetLastError();
}

cudaError_t chemistry(const DevicePtrs& p, int level, cudaStream_t s) {
  swk::ChemArgs<R> a;
  a.order = p.order;
  a.ctl = p.ctl;
  a.current_level = level;
  a.D = p.D;
  a.Dp = p.Dp;
  a.incoming = static_cast<const R*>(p.incoming);
  a.periodic = static_cast<const R*>(p.periodic);
  a.rate_scale = p.rate_scale;
  a.source = p.source;
  a.density = p.density;
  a.volume = p.volume;
  a.size = p.size;
  a.level = p.level;
  a.xhii = p.xhii;
  a.yneu = p.yneu;
  a.temperature = p.temperature;
  a.previous_rate = p.previous_rate;
  a.change_timescale = p.change_timescale;
  a.species_timestep = p.species_timestep;
  a.max_timestep = p.max_timestep;
  a.threshold = p.threshold;
  a.safety = p.chem_safety;
  a.scale_factor = p.scale_factor;
  a.prevent_cooling = p.prevent_cooling;
  swk::k_chemistry<R, kCarry><<<grid_for(p.num_cells, 128), 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t photon_rate(const DevicePtrs& p, double* out, cudaStream_t s) {
  swk::k_photon_rate<R><<<grid_for(p.num_cells, 256), 256, 0, s>>>(
      (uint32_t)p.num_cells, static_cast<const R*>(p.incoming), p.D, p.Dp, p.rate_scale, out);
  return cudaGetLastError();
}

cudaError_t export_rates(const DevicePtrs& p, const void* src, double* out, cudaStream_t s) {
  swk::k_export_rates<R><<<grid_for(p.num_cells * p.D, 256), 256, 0, s>>>(
      (uint32_t)p.num_cells, static_cast<const R*>(src), p.D, p.Dp, p.rate_scale, out);
  return cudaGetLastError();
}

}  // namespace

extern const PrecisionOps SWK_OPS = {
    SWK_NAME,    (int)sizeof(R), occupancy,  attenuation,  init_counts,
    sweep,       fold_periodic,  chemistry,  photon_rate,  export_rates,
};

}  // namespace swh
