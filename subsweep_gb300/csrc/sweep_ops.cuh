// Launchers of the precision-dependent kernels.  Included once by sweep_fp64.cu
// (R = double, reference-exact neutral fraction) and once by sweep_mixed.cu
// (R = float, carried neutral fraction); each defines SWK_R, SWK_CARRY and SWK_OPS.
#pragma once

#include <cmath>
#include <cstdlib>

#include "launch.h"
#include "sweep_device.cuh"
#if SWK_PULL
#include "sweep_pull.cuh"
#include "sweep_pull_setup.cuh"
#include "sweep_pull_lockstep.cuh"
#include "sweep_pull_wavefront.cuh"
#include "sweep_pull_geometry.cuh"
#include "sweep_pull_fold.cuh"
#else
#include "sweep_push_records.cuh"
#endif

namespace swh {
namespace {

using R = SWK_R;
constexpr bool kCarry = SWK_CARRY;

swk::SweepArgs<R> sweep_args(const DevicePtrs& p, int level) {
  swk::SweepArgs<R> a;
  a.off = p.off;
  a.geo32 = static_cast<const float4*>(p.geo32);
  a.geo64 = static_cast<const swk::Geo64*>(p.geo64);
  a.nbr = p.nbr;
  a.dir64 = p.dir64;
  a.dir32 = p.dir32;
  a.D = p.D;
  a.Np = p.Np;
  a.N = (uint32_t)p.num_cells;
  a.guard = p.guard;
  a.level = p.level;
  a.src_dir = static_cast<const R*>(p.src_dir);
  a.att = p.att;
  a.threshold = (R)(p.threshold / p.rate_scale);
  a.incoming = static_cast<R*>(p.incoming);
  a.outgoing = static_cast<R*>(p.outgoing);
  a.periodic = static_cast<R*>(p.periodic);
  a.pending = static_cast<R*>(p.pending);
  a.counters = p.counters;
  a.queue = p.queue;
  a.ctl = p.ctl;
  a.current_level = level;
  a.timeout_ns = p.timeout_ns;
  return a;
}

int grid_for(int64_t work, int block) {
  int64_t g = (work + block - 1) / block;
  if (g < 1) g = 1;
  if (g > 152 * 32) g = 152 * 32;
  return (int)g;
}

cudaError_t occupancy(int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, swk::k_sweep<R>, swk::kSweepThreads, 0);
}

// Whether the handle runs the staged wavefront kernel (pull variant 78), whose
// per-position periodic sources the fold then maintains.  The variant of a handle is
// fixed at creation (the autotuner's candidates do not include it).
bool staged_inputs(const DevicePtrs& p) {
  if (!p.per_pos) return false;
  int v = p.pull_variant;
  if (v <= 0)
    if (const char* env = std::getenv("SUBSWEEP_PULL_VARIANT")) v = std::atoi(env);
  return v == 78;
}

cudaError_t attenuation(const DevicePtrs& p, int level, cudaStream_t s) {
  swk::k_attenuation<kCarry><<<grid_for(p.num_cells, 256), 256, 0, s>>>(
      (uint32_t)p.num_cells, p.level, level, p.density, p.xhii, p.yneu, p.size, p.att, p.cell_sweep,
      p.epoch_base, p.epoch, static_cast<uint2*>(p.cellpack), static_cast<const float*>(p.src_dir));
  return cudaGetLastError();
}

cudaError_t init_counts(const DevicePtrs& p, int level, uint8_t* debug_counts, bool enqueue, cudaStream_t s) {
  swk::SweepArgs<R> a = sweep_args(p, level);
  swk::DirParam dirs;
  for (int i = 0; i < 3 * p.D; ++i) dirs.v[i] = p.dir32_host[i];
  const unsigned long long capacity = enqueue ? (unsigned long long)p.D * p.Np : 0ull;
  const int blocks = (int)((p.num_cells + swk::kCountThreads - 1) / swk::kCountThreads);
  swk::k_init_counts<R><<<blocks, swk::kCountThreads, 0, s>>>(a, dirs, capacity, debug_counts);
  return cudaGetLastError();
}

cudaError_t sweep(const DevicePtrs& p, int level, cudaStream_t s) {
  swk::SweepArgs<R> a = sweep_args(p, level);
  void* args[] = {&a};
  return cudaLaunchCooperativeKernel((const void*)swk::k_sweep<R>, dim3(p.coop_blocks), dim3(swk::kSweepThreads),
                                     args, 0, s);
}

cudaError_t occupancy_levels(int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, swk::k_sweep_sched<R>, swk::kLevelThreads, 0);
}

// The levelled push transport: over the precomputed downwind fractions when the grid
// has them, else computing the geometry on the fly.
cudaError_t sweep_levels(const DevicePtrs& p, int level, cudaStream_t s) {
  swk::SweepArgs<R> a = sweep_args(p, level);
  uint32_t total = (uint32_t)(p.num_cells * p.D);
#if !SWK_PULL
  if (p.push_rec) {
    const uint4* rec = static_cast<const uint4*>(p.push_rec);
    const uint32_t* tgt = p.push_tgt;
    const double* frac = p.push_frac;
    int bps = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, swk::k_sweep_sched_rec<R>,
                                                                  swk::kLevelThreads, 0);
    if (e != cudaSuccess) return e;
    if (p.level_bps_cap >= 1 && p.level_bps_cap < bps) bps = p.level_bps_cap;
    void* args[] = {&a, &rec, &total, &tgt, &frac};
    return cudaLaunchCooperativeKernel((const void*)swk::k_sweep_sched_rec<R>, dim3(bps * p.num_sms),
                                       dim3(swk::kLevelThreads), args, 0, s);
  }
#endif
  const uint32_t* order = p.order;
  void* args[] = {&a, &order, &total};
  return cudaLaunchCooperativeKernel((const void*)swk::k_sweep_sched<R>, dim3(p.level_blocks),
                                     dim3(swk::kLevelThreads), args, 0, s);
}

#if !SWK_PULL
// push path, once per grid: phase 0 writes the records' counts and the 64-bit scan of
// the chunk totals into `scratch` (total at scratch[num_chunks]); phase 1, with
// push_tgt / push_frac allocated, the offsets and the slots.
cudaError_t push_records(const DevicePtrs& p, int phase, unsigned long long* scratch, cudaStream_t s) {
  swk::SweepArgs<R> a = sweep_args(p, 0);
  uint4* rec = static_cast<uint4*>(p.push_rec);
  const uint32_t total = (uint32_t)(p.num_cells * p.D);
  const uint32_t nc = (total + swk::kCompactChunk - 1) / swk::kCompactChunk;
  if (phase == 0) {
    swk::k_push_rec_count<R><<<grid_for(p.num_cells * p.D, 256), 256, 0, s>>>(a, p.order, total, rec);
    swk::k_push_chunk_sums<R><<<nc, swk::kCompactThreads, 0, s>>>(rec, total, p.chunk);
    swk::k_push_scan64<R><<<1, 1024, 0, s>>>(p.chunk, nc, scratch);
  } else {
    swk::k_push_slots<R><<<nc, swk::kCompactThreads, 0, s>>>(a, rec, total, scratch, p.push_tgt, p.push_frac);
  }
  return cudaGetLastError();
}
#endif

// Seed of the schedule: dependency counts with every cell active (the caller has set
// all levels >= 0), tasks without dependencies appended to `order`.
cudaError_t schedule_seed(const DevicePtrs& p, cudaStream_t s) {
  swk::SweepArgs<R> a = sweep_args(p, 0);
  a.queue = p.order;
  swk::DirParam dirs;
  for (int i = 0; i < 3 * p.D; ++i) dirs.v[i] = p.dir32_host[i];
  const unsigned long long capacity = (unsigned long long)p.D * p.Np;
  const int blocks = (int)((p.num_cells + swk::kCountThreads - 1) / swk::kCountThreads);
  swk::k_init_counts<R><<<blocks, swk::kCountThreads, 0, s>>>(a, dirs, capacity, nullptr);
  return cudaGetLastError();
}

cudaError_t kahn_round(const DevicePtrs& p, uint32_t begin, uint32_t end, uint16_t* task_level, uint32_t round,
                       cudaStream_t s) {
  swk::SweepArgs<R> a = sweep_args(p, 0);
  const unsigned long long capacity = (unsigned long long)p.D * p.Np;
  swk::k_kahn_round<R><<<grid_for((int64_t)(end - begin), 256), 256, 0, s>>>(a, p.order, begin, end, capacity,
                                                                              task_level, round);
  return cudaGetLastError();
}

cudaError_t fold_periodic(const DevicePtrs& p, cudaStream_t s) {
  if (p.n_periodic_cells == 0) return cudaSuccess;
  swk::k_fold_periodic<R><<<grid_for((int64_t)p.n_periodic_cells * p.D, 256), 256, 0, s>>>(
      static_cast<R*>(p.periodic), static_cast<R*>(p.pending), p.periodic_cells, p.n_periodic_cells, p.D, p.Np);
  return cudaGetLastError();
}

cudaError_t chemistry(const DevicePtrs& p, int level, cudaStream_t s) {
  swk::ChemArgs<R> a;
  a.n = (uint32_t)p.num_cells;
  a.ctl = p.ctl;
  a.current_level = level;
  a.D = p.D;
  a.Np = p.Np;
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
  // FP32 transport: 2^-120 of the stored rate unit (normal FP32, full 24-bit precision,
  // 6 binary orders above the subnormal range; the unit is 2^(e - 96) of the total
  // source, so the floor is ~1e-65 of the total luminosity)
  a.rate_floor = sizeof(R) == 4 ? std::ldexp(1.0, -120) * p.rate_scale : 0.0;
  a.safety = p.chem_safety;
  a.scale_factor = p.scale_factor;
  a.prevent_cooling = p.prevent_cooling;
  swk::k_chemistry<R, kCarry><<<grid_for(p.num_cells, 128), 128, 0, s>>>(a);
  return cudaGetLastError();
}

#if SWK_PULL
swk::PullArgs pull_args(const DevicePtrs& p, int level) {
  swk::PullArgs a;
  a.off = p.off;
  a.geo16 = static_cast<const uint4*>(p.geo16);
  a.geo64 = static_cast<const swk::Geo64*>(p.geo64);
  a.dir64 = p.dir64;
  a.dir32 = p.dir32;
  a.D = p.D;
  a.Np = p.Np;
  a.N = (uint32_t)p.num_cells;
  a.level = p.level;
  a.src_dir = static_cast<const float*>(p.src_dir);
  a.att = p.att;
  a.threshold = (float)(p.threshold / p.rate_scale);
  a.periodic = static_cast<const float*>(p.periodic);
  a.qe = p.qe;
  a.inc = static_cast<float*>(p.incoming);
  a.ctl = p.ctl;
  a.current_level = level;
  a.epoch = p.epoch;
  a.epoch_base = p.epoch_base;
  a.cell_sweep = p.cell_sweep;
  a.timeout_ns = p.timeout_ns;
  a.rec = static_cast<const uint4*>(p.pull_rec);
  a.slots = static_cast<const uint2*>(p.pull_slots);
  a.act = nullptr;
  a.act_count = nullptr;
  a.count = (uint32_t)(p.num_cells * p.D);
  a.lvl = p.lvl;
  a.num_sched = p.num_sched_levels;
  a.cellpack = static_cast<const uint2*>(p.cellpack);
  a.per_pos = p.per_pos;
  a.pos_of_task = p.pos_of_task;
  a.order = p.order;
  return a;
}

uint32_t num_chunks(const DevicePtrs& p) {
  return (uint32_t)((p.num_cells * p.D + swk::kCompactChunk - 1) / swk::kCompactChunk);
}

cudaError_t records(const DevicePtrs& p, int phase, unsigned long long* chunk_off, cudaStream_t s) {
  if (p.geo_mode) {  // compact state: no records or slots; the fold's periodic entries, space by space
    if (phase != 1 || p.n_periodic_cells == 0) return cudaSuccess;
    for (int sp = 0; sp < p.num_spaces; ++sp) {
      const DevicePtrs v = space_view(p, sp);
      swk::k_fold_build<<<grid_for((int64_t)v.n_periodic_cells * v.D, 256), 256, 0, s>>>(
          pull_args(v, 0), v.periodic_cells, v.n_periodic_cells, v.fold_cnt, static_cast<uint2*>(v.fold_slots));
    }
    return cudaGetLastError();
  }
  swk::PullArgs a = pull_args(p, 0);
  uint4* rec = static_cast<uint4*>(p.pull_rec);
  const uint32_t nc = num_chunks(p);
  if (phase == 0) {
    swk::k_invert_order<<<grid_for(p.num_cells * p.D, 256), 256, 0, s>>>(p.order, a.count, p.pos_of_task);
    swk::k_pull_rec_count<<<grid_for(p.num_cells * p.D, 256), 256, 0, s>>>(a, p.order, a.count, rec);
    swk::k_pull_slot_chunks<<<nc, swk::kCompactThreads, 0, s>>>(rec, a.count, p.chunk);
    swk::k_scan_chunks64<<<1, swk::kScanThreads, 0, s>>>(p.chunk, nc, chunk_off);
  } else {
    swk::k_pull_slots<<<nc, swk::kCompactThreads, 0, s>>>(a, rec, a.count, chunk_off,
                                                          static_cast<uint2*>(p.pull_slots));
    if (p.n_periodic_cells > 0)
      swk::k_fold_build<<<grid_for((int64_t)p.n_periodic_cells * p.D, 256), 256, 0, s>>>(
          a, p.periodic_cells, p.n_periodic_cells, p.fold_cnt, static_cast<uint2*>(p.fold_slots));
  }
  return cudaGetLastError();
}

// Variants of the pull kernel: the warp-lockstep kernel with its shape as parameters
// (100 * prefetch depth (3: the next slots into L1 only) + 10 * lanes per task (2, 4, 8,
// or 6 for 16) + blocks per SM, + 1000 with streaming loads of records and slots, + 2000
// with the next block's words loaded one block ahead (prefetch depth 2); 83 and 84 name
// 183 and 184) and the level-synchronous wavefronts (72: registers, 78: TMA-staged).  SUBSWEEP_PULL_VARIANT picks one.

const void* pull_kernel(int variant) {
  switch (variant) {
    case 83:
    case 183: return (const void*)swk::k_sweep_pull_lockg<3, 8, 1>;
    case 84:
    case 184: return (const void*)swk::k_sweep_pull_lockg<4, 8, 1>;
    case 122: return (const void*)swk::k_sweep_pull_lockg<2, 2, 1>;
    case 123: return (const void*)swk::k_sweep_pull_lockg<3, 2, 1>;
    case 322: return (const void*)swk::k_sweep_pull_lockg<2, 2, 3>;
    case 323: return (const void*)swk::k_sweep_pull_lockg<3, 2, 3>;
    case 143: return (const void*)swk::k_sweep_pull_lockg<3, 4, 1>;
    case 144: return (const void*)swk::k_sweep_pull_lockg<4, 4, 1>;
    case 164: return (const void*)swk::k_sweep_pull_lockg<4, 16, 1>;
    case 242: return (const void*)swk::k_sweep_pull_lockg<2, 4, 2>;
    case 264: return (const void*)swk::k_sweep_pull_lockg<4, 16, 2>;
    case 283: return (const void*)swk::k_sweep_pull_lockg<3, 8, 2>;
    case 343: return (const void*)swk::k_sweep_pull_lockg<3, 4, 3>;
    case 344: return (const void*)swk::k_sweep_pull_lockg<4, 4, 3>;
    case 384: return (const void*)swk::k_sweep_pull_lockg<4, 8, 3>;
    case 1084: return (const void*)swk::k_sweep_pull_lockg<4, 8, 1, true>;
    case 1143: return (const void*)swk::k_sweep_pull_lockg<3, 4, 1, true>;
    case 1242: return (const void*)swk::k_sweep_pull_lockg<2, 4, 2, true>;
    case 1344: return (const void*)swk::k_sweep_pull_lockg<4, 4, 3, true>;
    case 2242: return (const void*)swk::k_sweep_pull_lockg<2, 4, 2, false, true>;
    case 2283: return (const void*)swk::k_sweep_pull_lockg<3, 8, 2, false, true>;
    case 72: return (const void*)swk::k_sweep_pull_wave<2>;
    case 78: return (const void*)swk::k_sweep_pull_staged;
    default: return nullptr;
  }
}

// the variant in use: set on the handle (autotuner or SUBSWEEP_PULL_VARIANT), else the
// default; an unknown number selects the default
int pull_variant(const DevicePtrs* p = nullptr) {
  int v = kDefaultPullVariant;
  if (p && p->pull_variant > 0) {
    v = p->pull_variant;
  } else if (const char* env = std::getenv("SUBSWEEP_PULL_VARIANT")) {
    v = std::atoi(env);
  }
  return pull_kernel(v) ? v : kDefaultPullVariant;
}

// candidates of the autotuner: the lockstep kernel with 2 lanes per task at 2 target
// blocks per SM, with 4 lanes per task at 3, and at 4 with the next block's slots
// brought into L1 only.  Measured on the C4 generator (transport G tasks/s over whole
// steps, direction-grouped schedule): at 256^3 122 18.6, 323 17.6, 344 16.7, 322 16.3,
// 143 16.1, 1344 15.9, 84 10.3, 242 10.2; at 128^3 143 14.3, 122 14.0, 344 13.6, 1344
// 13.1, 323 12.6.  Only dense sweeps are trials and a step may offer a single one (its
// first), so three candidates finish within three steps.
constexpr int kTuneVariants[] = {122, 143, 344};

// cooperative grid of a kernel: its occupancy limit (capped by
// SUBSWEEP_LEVEL_BLOCKS_PER_SM) on every SM
cudaError_t coop_grid(const DevicePtrs& p, const void* fn, int* grid, int threads = swk::kPullThreads) {
  int bps = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fn, threads, 0);
  if (e != cudaSuccess) return e;
  if (bps < 1) return cudaErrorInvalidConfiguration;
  if (p.level_bps_cap >= 1 && p.level_bps_cap < bps) bps = p.level_bps_cap;
  *grid = bps * p.num_sms;
  return cudaSuccess;
}

cudaError_t occupancy_pull(int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, pull_kernel(pull_variant()),
                                                       swk::kPullThreads, 0);
}

// Sparse sweeps (chosen by the host: above level 0 with fewer than half of the cells
// active) visit only the positions of active cells, from a stable compaction of the
// schedule built at the level's first sweep of a step (three launches; the kernel reads
// the count from the device).  Dense sweeps visit every position; the kernel stamps the
// inactive tasks itself.
// Shared memory of the staged wavefront kernel: the largest slot stages that fit the
// device's per-block limit next to the record, periodic and level-offset buffers;
// cudaErrorInvalidConfiguration when a stage would hold fewer than 9 slots per thread
// (the level offsets of a very deep schedule take the room).
cudaError_t staged_layout(const DevicePtrs& p, uint32_t* cap, size_t* smem) {
  int optin = 0;
  cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, 0);
  if (e != cudaSuccess) return e;
  const size_t fixed = swk::stg_smem_bytes(0, p.lvl_words) + sizeof(swk::StgShared) + 1024;
  if ((size_t)optin <= fixed) return cudaErrorInvalidConfiguration;
  const uint32_t c = (uint32_t)(((size_t)optin - fixed) / 16) & ~1u;
  if (c < 9u * swk::kStgThreads) return cudaErrorInvalidConfiguration;
  *cap = c;
  *smem = swk::stg_smem_bytes(c, p.lvl_words);
  static size_t attr = 0;
  if (attr != *smem) {
    e = cudaFuncSetAttribute((const void*)swk::k_sweep_pull_staged, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)*smem);
    if (e != cudaSuccess) return e;
    attr = *smem;
  }
  return cudaSuccess;
}

// compact state: the geometry kernel over every position of every task space, one
// launch (segment k of all spaces between two grid barriers)
cudaError_t sweep_pull_geo(const DevicePtrs& p, int level, cudaStream_t s) {
  static_assert(swk::kGeoMaxSpaces >= kMaxSpaces, "a task space per entry");
  const void* fn = (const void*)swk::k_sweep_pull_geo<1>;
  int grid = 0;
  cudaError_t e = coop_grid(p, fn, &grid, swk::kGeoThreads);
  if (e != cudaSuccess) return e;
  swk::GeoArgs g{};
  g.a = pull_args(p, level);
  g.num_spaces = p.num_spaces;
  g.max_levels = 0;
  for (int sp = 0; sp < p.num_spaces; ++sp) {
    const DevicePtrs v = space_view(p, sp);
    swk::GeoSpace& x = g.sp[sp];
    x.order = v.order;
    x.lvl = v.lvl;
    x.num_levels = v.num_sched_levels;
    x.qe = v.qe;
    x.inc = static_cast<float*>(v.incoming);
    x.periodic = static_cast<const float*>(v.periodic);
    x.dir32 = v.dir32;
    x.dir64 = v.dir64;
    g.max_levels = std::max(g.max_levels, x.num_levels);
  }
  if (g.max_levels == 0) return cudaSuccess;
  e = cudaMemsetAsync(&p.ctl->head, 0, sizeof(p.ctl->head), s);  // barrier arrivals
  if (e != cudaSuccess) return e;
  void* args[] = {&g};
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(swk::kGeoThreads), args, 0, s);
}

cudaError_t sweep_pull(const DevicePtrs& p, int level, cudaStream_t s) {
  if (p.geo_mode) return sweep_pull_geo(p, level, s);
  swk::PullArgs a = pull_args(p, level);
  const int variant = pull_variant(&p);
  if (p.sparse_sweep) {
    uint32_t* act = p.act_lv[level];
    uint32_t* cnt = p.act_counts + level;
    if (!act) return cudaErrorInvalidValue;
    if (p.compact_now) {  // mark the active cells' positions, then compact the bitmap
      const uint32_t words = (a.count + 31) / 32;
      const uint32_t nb = (words + swk::kBitsThreads - 1) / swk::kBitsThreads;
      cudaError_t e = cudaMemsetAsync(p.act_bits, 0, (size_t)words * sizeof(uint32_t), s);
      if (e != cudaSuccess) return e;
      swk::k_mark_active<<<grid_for(p.num_cells, 256), 256, 0, s>>>(p.level, level, (uint32_t)p.num_cells, p.D,
                                                                      p.Np, p.pos_of_task, p.act_bits);
      swk::k_bits_count<<<nb, swk::kBitsThreads, 0, s>>>(p.act_bits, words, p.chunk);
      swk::k_compact_scan<<<1, swk::kScanThreads, 0, s>>>(p.chunk, nb, cnt);
      swk::k_bits_scatter<<<nb, swk::kBitsThreads, 0, s>>>(p.act_bits, words, p.chunk, act);
      e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    a.act = act;
    a.act_count = cnt;
  }
  // the wavefront kernels run dense sweeps over a levelled schedule only; sparse sweeps
  // run the handle's lockstep variant (which tests the upwind cells' levels) or the
  // default one
  const bool wave = variant >= 70 && variant < 80;
  int v = (wave && (p.sparse_sweep || p.num_sched_levels == 0)) ? kDefaultPullVariant : variant;
  const void* fn = pull_kernel(v);
  void* args[] = {&a};
  uint32_t cap = 0;
  size_t smem = 0;
  if (fn == (const void*)swk::k_sweep_pull_staged && (!p.per_pos || staged_layout(p, &cap, &smem) != cudaSuccess)) {
    (void)cudaGetLastError();
    v = kDefaultPullVariant;  // no room for the stages: the lockstep kernel
    fn = pull_kernel(v);
  }
  if (fn == (const void*)swk::k_sweep_pull_staged) {  // one block of 1024 threads per SM
    uint32_t words = p.lvl_words;
    void* sargs[] = {&a, &cap, &words};
    return cudaLaunchCooperativeKernel(fn, dim3(p.num_sms), dim3(swk::kStgThreads), sargs, smem, s);
  }
  int grid = 0;
  cudaError_t e = coop_grid(p, fn, &grid);
  if (e != cudaSuccess) return e;
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(swk::kPullThreads), args, 0, s);
}

cudaError_t fold_pull(const DevicePtrs& p, cudaStream_t s) {
  if (p.n_periodic_cells == 0) return cudaSuccess;
  swk::PullArgs a = pull_args(p, 0);
  if (!staged_inputs(p)) a.per_pos = nullptr;
  const dim3 grid((p.n_periodic_cells + 255) / 256, p.D);
  // after a sweep that left cells inactive, only entries next to an active cell
  uint8_t* changed = nullptr;
  if (p.active_cells < p.num_cells && p.fold_changed) {
    changed = p.fold_changed;
    swk::k_fold_mark<<<grid_for(p.n_periodic_cells, 256), 256, 0, s>>>(a, p.periodic_cells, p.n_periodic_cells,
                                                                        changed);
  }
  if (p.geo_mode) {  // compact state: the entries of each task space
    for (int sp = 0; sp < p.num_spaces; ++sp) {
      const DevicePtrs v = space_view(p, sp);
      swk::PullArgs av = pull_args(v, 0);
      av.per_pos = nullptr;
      swk::k_fold_pull<<<dim3(grid.x, v.D), 256, 0, s>>>(av, static_cast<float*>(v.periodic), v.periodic_cells,
                                                         v.n_periodic_cells, v.fold_cnt,
                                                         static_cast<const uint2*>(v.fold_slots), changed);
    }
    return cudaGetLastError();
  }
  swk::k_fold_pull<<<grid, 256, 0, s>>>(a, static_cast<float*>(p.periodic), p.periodic_cells, p.n_periodic_cells,
                                        p.fold_cnt, static_cast<const uint2*>(p.fold_slots), changed);
  return cudaGetLastError();
}

cudaError_t photon_rate(const DevicePtrs& p, uint32_t last_epoch, double* out, cudaStream_t s) {
  swk::PullArgs a = pull_args(p, 0);
  swk::k_photon_rate_pull<<<grid_for(p.num_cells, 128), 128, 0, s>>>(a, last_epoch, p.rate_scale, out);
  return cudaGetLastError();
}

cudaError_t cell_rates(const DevicePtrs& p, uint32_t last_epoch, double* out, cudaStream_t s) {
  swk::PullArgs a = pull_args(p, 0);
  swk::k_cell_rates_pull<<<grid_for(p.num_cells, 128), 128, 0, s>>>(a, last_epoch, p.rate_scale, out);
  return cudaGetLastError();
}

cudaError_t export_rates(const DevicePtrs& p, int which, uint32_t last_epoch, double* out, cudaStream_t s) {
  swk::PullArgs a = pull_args(p, 0);
  swk::k_export_pull<<<grid_for(p.num_cells * p.D, 256), 256, 0, s>>>(a, last_epoch, which, p.rate_scale, out);
  return cudaGetLastError();
}
#else
cudaError_t photon_rate(const DevicePtrs& p, uint32_t, double* out, cudaStream_t s) {
  swk::k_photon_rate<R><<<grid_for(p.num_cells, 256), 256, 0, s>>>(
      (uint32_t)p.num_cells, static_cast<const R*>(p.incoming), p.D, p.Np, p.rate_scale, out);
  return cudaGetLastError();
}

cudaError_t cell_rates(const DevicePtrs& p, uint32_t, double* out, cudaStream_t s) {
  swk::k_cell_rates<R><<<grid_for(p.num_cells, 256), 256, 0, s>>>(
      (uint32_t)p.num_cells, static_cast<const R*>(p.incoming), static_cast<const R*>(p.periodic),
      static_cast<const R*>(p.src_dir), p.D, p.Np, p.rate_scale, out);
  return cudaGetLastError();
}

cudaError_t export_rates(const DevicePtrs& p, int which, uint32_t, double* out, cudaStream_t s) {
  const void* src = which == 0 ? p.incoming : (which == 1 ? p.outgoing : p.periodic);
  swk::k_export_rates<R><<<grid_for(p.num_cells * p.D, 256), 256, 0, s>>>(
      (uint32_t)p.num_cells, static_cast<const R*>(src), p.D, p.Np, p.rate_scale, out);
  return cudaGetLastError();
}
#endif

}  // namespace

#if SWK_PULL
extern const PrecisionOps SWK_OPS = {
    SWK_NAME,       (int)sizeof(R), true,       occupancy,     attenuation, init_counts, sweep,
    occupancy_pull, sweep_pull,     kahn_round, schedule_seed, fold_pull,   chemistry,   photon_rate,
    export_rates,   records,        cell_rates, SWK_CARRY != 0,
    (int)(sizeof(kTuneVariants) / sizeof(int)), kTuneVariants, nullptr,
};
#else
extern const PrecisionOps SWK_OPS = {
    SWK_NAME,         (int)sizeof(R), false,      occupancy,     attenuation,   init_counts, sweep,
    occupancy_levels, sweep_levels,   kahn_round, schedule_seed, fold_periodic, chemistry,   photon_rate,
    export_rates,     nullptr,        cell_rates, SWK_CARRY != 0,
    0, nullptr,       push_records,
};
#endif

}  // namespace swh
