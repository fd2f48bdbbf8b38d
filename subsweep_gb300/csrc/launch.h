// Launch interface between the C++ host runtime (sweep_host.cpp) and the two
// kernel translation units: sweep_fp64.cu (FP64 drop-in, compiled without FMA
// contraction so every expression rounds as the reference's does) and
// sweep_mixed.cu (FP32 transport, FP64 chemistry, FMA allowed).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace swk {
struct SweepCtl;
}

namespace swh {

// Raw device pointers of one handle.  Rate arrays are double (FP64) or float (mixed).
struct DevicePtrs {
  int64_t num_cells;
  int D, Dp, words, num_levels;
  float guard;
  double rate_scale;         // photons/s per stored rate unit
  double threshold;          // significant_rate_threshold in photons/s
  double max_timestep, timestep_safety, chem_safety, scale_factor;
  int prevent_cooling;
  // geometry
  const long long* row_ptr;
  const void* geo64;  // {nx, ny, nz, area} x E doubles, 32-byte aligned
  const void* geo32;  // float4[E]
  const uint32_t* nbr;
  const double* size;
  const double* volume;
  const double* dir64;
  const float* dir32;
  // cells
  uint8_t* level;
  uint32_t* order;
  const double* density;
  const double* source;
  double* xhii;
  double* yneu;
  double* temperature;
  double* att;
  double* previous_rate;
  double* change_timescale;
  double* species_timestep;
  double* ionization_time;
  // tasks
  void* incoming;
  void* outgoing;
  void* periodic;
  void* pending;
  uint32_t* counters;
  uint32_t* ready;
  uint32_t* queued;
  uint32_t* frontier0;
  uint32_t* frontier1;
  const uint32_t* periodic_cells;
  uint32_t n_periodic_cells;
  swk::SweepCtl* ctl;
  int coop_blocks;
  unsigned long long timeout_ns;
  uint32_t max_rounds;
};

struct PrecisionOps {
  const char* name;
  int rate_bytes;
  // blocks of the persistent sweep kernel that are co-resident on this device
  cudaError_t (*occupancy)(int* blocks_per_sm);
  cudaError_t (*attenuation)(const DevicePtrs&, int level, cudaStream_t);
  cudaError_t (*init_counts)(const DevicePtrs&, int level, uint8_t* debug_counts, cudaStream_t);
  cudaError_t (*sweep)(const DevicePtrs&, int level, cudaStream_t);
  cudaError_t (*fold_periodic)(const DevicePtrs&, cudaStream_t);
  cudaError_t (*chemistry)(const DevicePtrs&, int level, cudaStream_t);
  cudaError_t (*photon_rate)(const DevicePtrs&, double* out, cudaStream_t);
  cudaError_t (*export_rates)(const DevicePtrs&, const void* src, double* out, cudaStream_t);
};

extern const PrecisionOps kOpsFP64;
extern const PrecisionOps kOpsMixed;

// Precision-independent kernels (compiled in sweep_fp64.cu).
cudaError_t launch_update_levels(const DevicePtrs&, int lowest_allowed, cudaStream_t);
cudaError_t launch_level_hist(const DevicePtrs&, cudaStream_t);
cudaError_t launch_level_order(const DevicePtrs&, cudaStream_t);
cudaError_t launch_ionization_time(const DevicePtrs&, double time, cudaStream_t);

}  // namespace swh
