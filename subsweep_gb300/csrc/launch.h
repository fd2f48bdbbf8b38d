// Launch interface between the C++ host runtime (sweep_host.cpp) and the two
// kernel translation units: sweep_fp64.cu (FP64 drop-in, compiled without FMA
// contraction so every expression rounds as the reference's does) and
// sweep_mixed.cu (FP32 transport, FP64 chemistry, FMA allowed).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/subsweep_gpu.h"

namespace swk {
struct SweepCtl;
}

namespace swh {

// Task spaces of the compact pull state: directions [space_d0[s], space_d0[s + 1]).
constexpr int kMaxSpaces = 8;

// Raw device pointers of one handle.  Rate arrays are double (FP64) or float (mixed);
// per-task arrays are [dir][cell] with cell stride Np.
struct DevicePtrs {
  int64_t num_cells;
  int D, num_levels;
  uint32_t Np;
  float guard;
  double rate_scale;         // photons/s per stored rate unit
  double threshold;          // significant_rate_threshold in photons/s
  double max_timestep, timestep_safety, chem_safety, scale_factor;
  int prevent_cooling;
  float dir32_host[128 * 3];  // directions for by-value kernel parameters
  // geometry
  const uint32_t* off;
  const void* geo64;  // {nx, ny, nz, area} x E doubles, 32-byte aligned
  const void* geo32;  // float4[E], area scaled by a power of two
  const void* geo16;  // uint4[E] {area*n (scaled) x3, nbr | kind << 30} (pull path)
  const uint32_t* nbr;
  const double* size;
  const double* volume;
  const double* dir64;
  const float* dir32;
  // cells
  uint8_t* level;
  const double* density;
  const double* source;
  const void* src_dir;       // source / D per cell in stored rate units (R)
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
  uint32_t* queue;
  unsigned long long* qe;    // pull path: {q, sweep number} and incoming rate per schedule position
  uint32_t epoch;            // pull path: number of the current level sweep
  const uint32_t* epoch_base; // graph replay: sweep numbers are *epoch_base + epoch
  uint32_t* cell_sweep;      // pull path: number of the last sweep that solved each cell
  void* cellpack;            // pull path: uint2 per cell {(float) attenuation or inactive mark, source / D}
  float* per_pos;            // pull path: periodic source of every schedule position
  uint32_t lvl_words;        // level offsets allocated (a multiple of 4, >= num_sched_levels + 1)
  uint32_t* order;           // levelled schedule: task ids grouped by Kahn level
  const uint32_t* lvl;       // level offsets into order [num_sched_levels + 1]
  uint32_t num_sched_levels; // 0: no levelled schedule (cyclic graph)
  void* push_rec;            // push path: uint4 record per schedule position (or null)
  uint32_t* push_tgt;        // push path: downwind targets (neighbour | kind << 30)
  double* push_frac;         // push path: downwind fractions eff / total (FP64)
  void* pull_rec;            // pull path: uint4 task record per schedule position
  void* pull_slots;          // pull path: uint2 upwind slots of all positions
  uint32_t* act_lv[32];      // pull path: compacted active positions per level (lazily allocated)
  uint32_t* act_counts;      // pull path: their lengths [32] (device)
  uint32_t* pos_of_task;     // pull path: schedule position of every task (inverse order)
  uint8_t* fold_cnt;         // pull path: upwind periodic faces per (periodic cell, direction)
  void* fold_slots;          // pull path: their uint2 {upwind schedule position, weight}, 4 per entry
  uint8_t* fold_changed;     // pull path: per periodic cell, a periodic neighbour was active
  uint32_t* act_bits;        // pull path: one bit per schedule position (sparse compaction)
  // pull path, compact state (geo_mode): no task records, upwind slots or inverse order
  // (pos_of_task is null and the words are indexed by task); the geometry kernel sweeps
  // every position of each task space (directions split so that a space holds fewer
  // than 2^31 tasks), one space after another, with its own levelled schedule
  int geo_mode;
  int num_spaces;                       // 1 unless geo_mode splits the directions
  int space_d0[kMaxSpaces + 1];
  uint32_t* space_lvl[kMaxSpaces];      // segment offsets of each space's schedule
  uint32_t space_segments[kMaxSpaces];
  uint32_t space_lvl_words[kMaxSpaces];
  int sparse_sweep;          // pull path: this launch runs over the compacted list of its level
  int compact_now;           // pull path: ... and builds that list first
  uint32_t* chunk;           // pull path: compaction chunk offsets, count at [num_chunks]
  int64_t active_cells;      // pull path: cells active in the sweep being launched
  int compact_mode;          // pull path: 0 by density, 1 always compact, 2 never (lockstep)
  int pull_variant;          // pull path: transport kernel variant (0: the default)
  int num_sms;
  int level_bps_cap;         // SUBSWEEP_LEVEL_BLOCKS_PER_SM, 0: each kernel's occupancy limit
  int level_blocks;          // resident blocks of the levelled kernel
  const uint32_t* periodic_cells;
  uint32_t n_periodic_cells;
  swk::SweepCtl* ctl;
  int coop_blocks;
  unsigned long long timeout_ns;
};

struct PrecisionOps {
  const char* name;
  int rate_bytes;
  bool pull;  // pull-form transport (mixed path): no counters, no queue
  // blocks of the persistent sweep kernel that are co-resident on this device
  cudaError_t (*occupancy)(int* blocks_per_sm);
  cudaError_t (*attenuation)(const DevicePtrs&, int level, cudaStream_t);
  cudaError_t (*init_counts)(const DevicePtrs&, int level, uint8_t* debug_counts, bool enqueue, cudaStream_t);
  cudaError_t (*sweep)(const DevicePtrs&, int level, cudaStream_t);
  cudaError_t (*occupancy_levels)(int* blocks_per_sm);
  cudaError_t (*sweep_levels)(const DevicePtrs&, int level, cudaStream_t);
  cudaError_t (*kahn_round)(const DevicePtrs&, uint32_t begin, uint32_t end, uint16_t* task_level, uint32_t round,
                            cudaStream_t);
  cudaError_t (*schedule_seed)(const DevicePtrs&, cudaStream_t);
  cudaError_t (*fold_periodic)(const DevicePtrs&, cudaStream_t);
  cudaError_t (*chemistry)(const DevicePtrs&, int level, cudaStream_t);
  // which: 0 incoming, 1 outgoing, 2 periodic; last_epoch: sweep number of the step's
  // last sweep (pull path)
  cudaError_t (*photon_rate)(const DevicePtrs&, uint32_t last_epoch, double* out, cudaStream_t);
  cudaError_t (*export_rates)(const DevicePtrs&, int which, uint32_t last_epoch, double* out, cudaStream_t);
  // pull path, once per grid: phase 0 writes the per-position task records and the
  // 64-bit exclusive scan of the upwind counts per chunk into chunk_off (total at
  // chunk_off[num_chunks]); phase 1, with pull_slots allocated, writes the slots.
  // nullptr on the push path.
  cudaError_t (*records)(const DevicePtrs&, int phase, unsigned long long* chunk_off, cudaStream_t);
  // rate of every cell summed over directions (incoming + source/D + periodic),
  // photons/s
  cudaError_t (*cell_rates)(const DevicePtrs&, uint32_t last_epoch, double* out, cudaStream_t);
  bool carry_neutral;  // the chemistry carries 1 - x_HII as its own state (yneu)
  // pull path: transport kernel variants the autotuner tries (count, ids); 0 on the push path
  int num_tune_variants;
  const int* tune_variants;
  // push path, once per grid: precomputed downwind fractions (phases as records);
  // nullptr on the pull path
  cudaError_t (*push_records)(const DevicePtrs&, int phase, unsigned long long* scratch, cudaStream_t);
};

// pull path: transport kernel variant used without autotuning (the lockstep kernel with
// 4 lanes per task, 3 target blocks per SM)
constexpr int kDefaultPullVariant = 143;

// The pointers of task space s of a compact pull state: its directions, its per-task
// arrays (incoming, periodic, words, counters: [dir][cell] slices; FP32 rates), its
// schedule and its periodic fold entries.  Task ids and positions inside a view are
// local to the space.  With one space the view is the handle's pointers.
inline DevicePtrs space_view(const DevicePtrs& p, int s) {
  if (p.num_spaces <= 1) return p;
  DevicePtrs v = p;
  const int d0 = p.space_d0[s];
  const size_t off = (size_t)d0 * p.Np;
  v.D = p.space_d0[s + 1] - d0;
  for (int i = 0; i < 3 * v.D; ++i) v.dir32_host[i] = p.dir32_host[3 * d0 + i];
  v.dir64 = p.dir64 + 3 * d0;
  v.dir32 = p.dir32 + 3 * d0;
  v.incoming = static_cast<char*>(p.incoming) + off * sizeof(float);
  v.periodic = static_cast<char*>(p.periodic) + off * sizeof(float);
  v.qe = p.qe + off;
  v.counters = p.counters + off / 4;  // u8 counters, four to a word (Np is a multiple of 32)
  v.order = p.order + (size_t)p.num_cells * d0;
  v.lvl = p.space_lvl[s];
  v.num_sched_levels = p.space_segments[s];
  v.lvl_words = p.space_lvl_words[s];
  constexpr size_t kFoldEntrySlots = 4;
  if (p.fold_cnt) v.fold_cnt = p.fold_cnt + (size_t)d0 * p.n_periodic_cells;
  if (p.fold_slots)
    v.fold_slots = static_cast<char*>(p.fold_slots) + (size_t)d0 * p.n_periodic_cells * kFoldEntrySlots * 8;
  v.num_spaces = 1;
  return v;
}

extern const PrecisionOps kOpsFP64;
extern const PrecisionOps kOpsMixed;

// Read access to a handle's device state for entry points defined outside the host
// runtime's translation unit.
struct HandleView {
  DevicePtrs* p;
  const PrecisionOps* ops;
  cudaStream_t stream;
  int device;
  int64_t num_cells;
  int num_directions;
  int num_levels;
};
bool handle_view(sw_handle* h, HandleView* out);
// Record an error message on the handle (returned by sw_last_error) and return `st`.
sw_status handle_fail(sw_handle* h, sw_status st, const char* message);
// Forget the handle's last error (every entry point starts with this).
void handle_clear_error(sw_handle* h);

// Makes a handle's device current for the duration of an entry point and makes the
// caller's device current again on return, so a host that drives other GPU work on
// another device keeps its own selection.  `status` is the result of the selection.
struct DeviceScope {
  int previous = -1;
  cudaError_t status = cudaSuccess;
  explicit DeviceScope(int device) {
    int current = -1;
    status = cudaGetDevice(&current);
    if (status == cudaSuccess && current != device) {
      status = cudaSetDevice(device);
      if (status == cudaSuccess) previous = current;
    }
  }
  ~DeviceScope() {
    if (previous >= 0) cudaSetDevice(previous);
  }
  DeviceScope(const DeviceScope&) = delete;
  DeviceScope& operator=(const DeviceScope&) = delete;
};

// Precision-independent kernels (compiled in sweep_fp64.cu).
cudaError_t launch_update_levels(const DevicePtrs&, int lowest_allowed, cudaStream_t);
cudaError_t launch_level_hist(const DevicePtrs&, cudaStream_t);
// `time_dev`, when given, is read on the device instead of `time` (graph replay)
cudaError_t launch_ionization_time(const DevicePtrs&, double time, cudaStream_t, const double* time_dev = nullptr);
// Time series from per-cell summed rates: `partial` holds kTimeSeriesPartials doubles,
// `out6` receives the six averages (device memory).
constexpr int kTimeSeriesPartials = 256 * 8;
cudaError_t launch_time_series(const DevicePtrs&, const double* cell_rate, bool carry_neutral, double* partial,
                               double* out6, cudaStream_t);

}  // namespace swh
